// Kernel launchers of the movement-sim per-tick path (implemented in msim_kernels.cu).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "msim_device.cuh"

namespace msim {

// Radix sort (onesweep: one global histogram pass, then one chained-scan pass per digit)
constexpr int kSortThreads = 256;
constexpr int kSortRows = 16;                               // items per thread
constexpr uint32_t kSortTile = kSortThreads * kSortRows;    // 4096 items per block
constexpr int kSortRowsDev = 4;                             // the same, for passes with a device-side count
constexpr uint32_t kRadix = 256;                            // 8-bit digits
constexpr int kMaxPasses = 3;                               // keys up to 24 bits
constexpr int kQueryThreads = 128;
constexpr int kStepThreads = 512;  // measured at 16 M: 0.122 ms per tick against 0.136 with 256
constexpr int kStepPer = 1;        // entities per thread and iteration of k_step
constexpr int kMoveThreads = 128;  // move-only multi-tick launches (k_move)
constexpr uint32_t kMaxCap = 256;
constexpr uint32_t kPairBins = 256;  // pair counters (summed on read), spread to avoid one hot atomic

// Entity state in slot order (structure of arrays)
struct EntityState {
    float2* pos;
    uint32_t* head;
    uint4* rng;
    float* speed;
    uint32_t* slot_id;  // entity id held by each slot
};

struct StepLaunch {
    DeviceMap map;
    EntityState st;
    uint32_t n;
    float dt;
    uint32_t ticks;       // 0: only keys/histogram of the current positions
    uint32_t rng_kind;
    uint32_t* key;        // nullptr: no spatial key
    uint32_t* hist;       // passes * 256 digit counts (accumulated)
    TileGrid grid;
    uint32_t passes;
    uint32_t* err;
    int blocks;           // grid size (grid-stride loop)
    // Host round trip with the caller's arrays both input and output: the headings and
    // RNG states that change are also written to them (device-mapped page-locked host
    // memory, indexed by id_base + slot; slot = entity id there), so only positions
    // need a download.  nullptr otherwise.
    uint32_t* host_head = nullptr;
    uint4* host_rng = nullptr;
    uint32_t id_base = 0;
    // Words the move step zeroes before its entities (nullptr / 0: none): the next
    // kernels' scratch, cleared here instead of by memsets that would sit between the
    // chained launches of the tick.
    uint32_t* zero_a = nullptr;
    uint32_t zero_a_words = 0;
    uint32_t* zero_b = nullptr;  // one word
    // Largest displacement of the tick (nullptr: not measured): every moved entity's
    // max(|x - x0|, |y - y0|) against index_pos (by slot, the positions the current
    // index was built from) is atomically maxed into *disp_max as float bits (a
    // non-finite displacement counts as +inf).
    const float2* index_pos = nullptr;
    uint32_t* disp_max = nullptr;
    // With disp_max: the first entity (id_base + slot) whose heading names a road out of
    // range is atomically min-ed into *first_bad (NULL: not checked here).
    uint32_t* first_bad = nullptr;
    // One move tick (move-only kernel): each moved position is also written to
    // rank_pos[rank[slot]] (its place in a sorted order of rank_n entries; larger ranks
    // are skipped).
    const uint32_t* rank = nullptr;
    float2* rank_pos = nullptr;
    uint32_t rank_n = 0;
};

cudaError_t launch_init_entities(cudaStream_t s, const DeviceMap& m, EntityState st, uint32_t n,
                                 uint32_t rng_kind, uint64_t seed, uint32_t placement, float smin,
                                 float smax);
cudaError_t launch_step(cudaStream_t s, const StepLaunch& a);
// Look-back bookkeeping that lets consecutive radix passes run without a memset
// between them: before its tiles a pass zeroes next_lookback[0, *next_dirty) and
// *next_ticket, and sets *my_dirty to the look-back words it publishes itself.  The
// look-back words and tickets start zeroed, and every pass over them is chained.
struct SweepChain {
    uint32_t* next_lookback = nullptr;
    uint32_t* next_ticket = nullptr;
    const uint32_t* next_dirty = nullptr;
    uint32_t* my_dirty = nullptr;
};
// Look-back words one pass over n items may publish (either tile size).
size_t sort_lookback_words(uint32_t n);
// Polls of a look-back word before a wait gives up (kErrTimeout): about a second.
constexpr uint32_t kDefaultSpinLimit = 1u << 24;
cudaError_t launch_onesweep(cudaStream_t s, const uint32_t* keys_in, const uint32_t* vals_in,
                            uint32_t* keys_out, uint32_t* vals_out, uint32_t n, uint32_t shift,
                            const uint32_t* digit_count, uint32_t* lookback, uint32_t* ticket,
                            uint32_t* err, const uint32_t* n_dev = nullptr,  // n_dev: count on the device (<= n)
                            const SweepChain* chain = nullptr, uint32_t spin_limit = kDefaultSpinLimit);
cudaError_t launch_ranges(cudaStream_t s, const uint32_t* sorted_key, uint32_t n, uint2* ranges, uint32_t num_keys,
                          uint32_t ybits = 0);
// Key-start table of sorted keys (num_keys + 1 entries).  chunks / chunk_count
// (kstart_chunks(num_keys) uint4 entries and one counter; may be NULL) enable the
// per-position kernel, which also gathers pos into sorted order (sorted_pos, n entries)
// when sorted_slot, pos and sorted_pos are given.  *kernels (may be NULL) receives the
// number of kernels launched.
uint32_t kstart_chunks(uint64_t num_keys);
cudaError_t launch_kstart(cudaStream_t s, const uint32_t* sorted_key, uint32_t n, uint32_t* kstart, uint32_t num_keys,
                          uint4* chunks = nullptr, uint32_t* chunk_count = nullptr, uint32_t* kernels = nullptr,
                          const uint32_t* sorted_slot = nullptr, const float2* pos = nullptr,
                          float2* sorted_pos = nullptr, const uint32_t* err = nullptr);
cudaError_t launch_query(cudaStream_t s, uint32_t cap, const uint32_t* kstart, const uint32_t* sorted_slot,
                         const float2* sorted_pos, const uint32_t* slot_id, TileGrid grid, uint32_t n, uint32_t* count,
                         uint32_t* list, unsigned long long* pair_bins,  // pair_bins: kPairBins counters
                         const uint32_t* err = nullptr,  // err: the status word (skip after a failed wait)
                         // count_by_id (may be NULL; only when slot = entity id): every count also
                         // written at its entity's id
                         uint32_t* count_by_id = nullptr);
// Incremental index update: split the previous sorted order P (keys PK; P[q] = q when
// identity) by whether the new key NK[slot] changed (A: unchanged, B: changed; counts
// -> counts[0..1]; B's digit counts -> hist), then, after B is sorted, merge A and B
// into out_key / out_val, writing the key-start table and the sorted positions.
// changed_total (may be NULL) accumulates |B| (entries that go through the sort).
// lookback (mark_tiles(n) words), ticket and hist must be zero when the split starts.
uint32_t mark_tiles(uint32_t n);
uint32_t merge_tiles(uint32_t n);
cudaError_t launch_mark(cudaStream_t s, const uint32_t* P, bool identity, const uint32_t* PK, const uint32_t* NK,
                        uint32_t n, uint32_t passes, uint32_t* a_key, uint32_t* a_val, uint32_t* b_key,
                        uint32_t* b_val, uint32_t* hist, unsigned long long* lookback, uint32_t* ticket,
                        uint32_t* counts, uint32_t* err, unsigned long long* changed_total = nullptr,
                        uint32_t spin_limit = kDefaultSpinLimit);
// chunk_count_zeroed: the long-gap counter was already zeroed in the tick (else a
// memset does it first).  sorted_pos NULL: no positions are gathered (pos unused).
cudaError_t launch_merge(cudaStream_t s, const uint32_t* a_key, const uint32_t* a_val, const uint32_t* b_key,
                         const uint32_t* b_val, const uint32_t* counts, uint32_t* split, uint32_t n,
                         uint32_t* out_key, uint32_t* out_val, const float2* pos, float2* sorted_pos,
                         uint32_t* kstart, uint32_t num_keys, uint4* chunks, uint32_t* chunk_count, uint32_t* err,
                         uint32_t* kernels, bool chunk_count_zeroed = false,
                         uint32_t* rank = nullptr);  // rank (may be NULL): rank[out_val[p]] = p
// out[q] = pos[P[q]] for the q whose slot P[q] lies in [lo, lo + cnt) (q < n; the
// other entries are left as they are): the positions of one uploaded chunk of a host
// tick copied to their places in the sorted order P.
cudaError_t launch_gather_chunk(cudaStream_t s, const uint32_t* P, uint32_t n, uint32_t lo, uint32_t cnt,
                                const float2* pos, float2* out);
// out[0] = largest |speed|, out[1] = largest |x| or |y| of the n entities, as float
// bits (atomically maxed: out must hold zeros; NaN or infinite values count as +inf).
cudaError_t launch_bounds(cudaStream_t s, const float* speed, const float2* pos, uint32_t n, uint32_t* out);
cudaError_t launch_iota(cudaStream_t s, uint32_t* out, uint32_t n);
// *first_bad = first i with (head[i] & road mask) >= num_roads, or 0xffffffff
cudaError_t launch_check_roads(cudaStream_t s, const uint32_t* head, uint32_t n, uint32_t num_roads,
                               uint32_t* first_bad);
// The same over entities [first, first + n) without resetting *first_bad (atomic min).
cudaError_t launch_check_roads_range(cudaStream_t s, const uint32_t* head, uint32_t first, uint32_t n,
                                     uint32_t num_roads, uint32_t* first_bad);
cudaError_t launch_fill(cudaStream_t s, float* out, uint32_t n, float v);
// With kErrTimeout in *err (may be NULL) the state is copied in its current order.
cudaError_t launch_permute(cudaStream_t s, const uint32_t* sorted_slot, EntityState src,
                           EntityState dst, uint32_t n, const uint32_t* err = nullptr);
cudaError_t launch_export_state(cudaStream_t s, EntityState st, uint32_t n, float2* pos,
                                uint32_t* head, uint4* rng, float* speed);
cudaError_t launch_export_neighbours(cudaStream_t s, const uint32_t* sorted_slot, const uint32_t* slot_id,
                                     const uint32_t* count, const uint32_t* list, uint32_t n,
                                     uint32_t cap, uint32_t* out_count, uint32_t* out_idx);
cudaError_t launch_export_aos(cudaStream_t s, const DeviceMap& m, EntityState st, uint32_t n, float dt,
                              const uint32_t* sorted_slot, const uint32_t* count, void* out);

cudaError_t configure_kernels(uint32_t cap);
int step_blocks_for(int device, uint32_t n);

}  // namespace msim
