// CUDA kernels of the movement-sim per-tick path for sm_103a.
//
// Per neighbour tick (entity state is kept in "slot" order, i.e. the spatial
// order of the last re-ordering):
//   k_step      move every entity one tick (random_move.comp:869-874), write its
//               tile Morton key and count the key's radix digits (warp-aggregated
//               by ballot over runs of equal digits, one shared atomic per run)
//   k_onesweep  one stable LSD radix pass per 8-bit digit (decoupled look-back,
//               warp-level multi-split ranking with __match_any_sync; every block
//               scans the pass's digit counts into offsets itself)
//   k_kstart    key-start table: first sorted position of every key (tile + band)
//   k_query     radius neighbour query (random_move.comp:541-719 semantics: the
//               pair predicate of :551-562), count + the cap smallest ids
// After the first neighbour tick the sort is replaced by an incremental update of the
// previous order (msim_incsort.cuh): k_mark splits it by changed keys, k_onesweep
// sorts the changed entries, k_merge_path + k_merge merge them back and write the
// key-start table and the sorted positions.
// Every few ticks k_permute re-orders the entity state by the sorted order so
// that the step and the query keep reading memory almost sequentially.
#include <algorithm>
#include <cstdio>

#include "msim_kernels.cuh"

namespace msim {
namespace {

constexpr uint32_t kFlagAgg = 0x40000000u;
constexpr uint32_t kFlagPrefix = 0x80000000u;
constexpr uint32_t kFlagMask = 0xc0000000u;
constexpr uint32_t kValueMask = 0x3fffffffu;
// polls of a look-back word before a wait gives up with kErrTimeout: the per-context
// limit (msim_set_wait_limit) defaults to kDefaultSpinLimit, about a second
constexpr int kLookBack = 4;               // predecessor tiles read per look-back round of a radix pass

// Kernels of the per-tick chain (move, split, radix passes, merge, key-start fill,
// re-ordering) are launched with programmatic stream serialisation: a chain kernel
// lets the next one launch once all its own blocks run, and waits for its
// predecessor to finish, with its writes visible, before it touches global memory.
// Only the launch and block dispatch overlap the predecessor's tail.  A dependent is
// launched only when every block of its predecessor is resident, so waiting blocks
// never keep a predecessor's block from being scheduled.
__device__ __forceinline__ void chain_enter() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}
__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// After a bounded wait has given up (kErrTimeout in the status word) the index of
// the tick is incomplete: every later kernel that reads it returns without work
// (k_permute copies the state in its current order), so no kernel consumes a partial
// sort until the host has read and cleared the status and rebuilt the index.
__device__ __forceinline__ bool index_failed(const uint32_t* err) {
    return err != nullptr && (ld_relaxed(err) & kErrTimeout) != 0u;
}

// Block-wide exclusive sum over NT threads; s_warp needs NT/32 + 1 words.
// All threads must call it; returns the exclusive prefix, *total = block sum.
template <int NT>
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_warp, uint32_t* total) {
    constexpr int NW = NT / 32;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (uint32_t)NW ? s_warp[lane] : 0u;
        uint32_t incl = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= (uint32_t)o) incl += y;
        }
        if (lane < (uint32_t)NW) s_warp[lane] = incl - w;
        if (lane == (uint32_t)NW - 1) s_warp[NW] = incl;
    }
    __syncthreads();
    uint32_t r = s_warp[warp] + x - v;
    if (total) *total = s_warp[NW];
    __syncthreads();
    return r;
}

__device__ __forceinline__ uint4 pcg32_seed(uint64_t initstate, uint64_t initseq) {
    uint64_t inc = (initseq << 1) | 1u;
    uint4 s = make_uint4(0u, 0u, (uint32_t)inc, (uint32_t)(inc >> 32));
    (void)pcg32_next(s);
    uint64_t st = (((uint64_t)s.y << 32) | s.x) + initstate;
    s.x = (uint32_t)st;
    s.y = (uint32_t)(st >> 32);
    (void)pcg32_next(s);
    return s;
}

// Deterministic initializer (replaces Simulator.cpp:114-129, Entity.cpp:44-49):
// draw streams 1 road, 2 fraction along the road, 3 speed, 4/5 RNG state.
__global__ void k_init(DeviceMap m, EntityState st, uint32_t n, uint32_t rng_kind, uint64_t seed,
                       uint32_t placement, float smin, float smax) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint64_t dr = d_draw(seed, 1, i);
        uint32_t r = (uint32_t)(((dr >> 32) * (uint64_t)m.num_roads) >> 32);
        float4 rp = m.road_pos[r];
        float px = rp.x, py = rp.y;
        if (placement == 1) {
            float u = unit24(d_draw(seed, 2, i));
            px = __fadd_rn(rp.x, __fmul_rn(u, __fsub_rn(rp.z, rp.x)));
            py = __fadd_rn(rp.y, __fmul_rn(u, __fsub_rn(rp.w, rp.y)));
        }
        st.pos[i] = make_float2(px, py);
        st.head[i] = r | kHeadToEnd;
        float v = unit24(d_draw(seed, 3, i));
        st.speed[i] = __fadd_rn(smin, __fmul_rn(v, __fsub_rn(smax, smin)));
        uint64_t a = d_draw(seed, 4, i);
        uint64_t b = d_draw(seed, 5, i);
        uint4 s;
        if (rng_kind == 1) {
            s = pcg32_seed(a, b);
        } else {
            s = make_uint4((uint32_t)a, (uint32_t)(a >> 32), (uint32_t)b, (uint32_t)(b >> 32));
            if ((s.x | s.y | s.z | s.w) == 0u) s.x = 1u;
        }
        st.rng[i] = s;
        st.slot_id[i] = i;
    }
}

// Move `ticks` ticks (state kept in registers across ticks), then optionally
// write the tile key and accumulate the radix digit histograms of all passes.
template <int RNG, bool KEY>
__device__ __forceinline__ void digit_counts(uint32_t key, bool valid, uint32_t lane, uint32_t passes,
                                             uint32_t* s_hist) {
    // Warp-aggregated digit counts.  Slots follow the spatial order of the last
    // re-ordering, so neighbouring lanes mostly share digits: each run of equal
    // digits among consecutive lanes adds its length with one shared atomic, issued
    // by the run's first lane (found by ballot).
    const unsigned vm = __ballot_sync(0xffffffffu, valid);
    for (uint32_t ps = 0; ps < passes; ps++) {
        const uint32_t d = (key >> (8u * ps)) & 0xffu;
        const uint32_t dprev = __shfl_up_sync(0xffffffffu, d, 1);
        const bool head = valid && (lane == 0 || d != dprev);
        const unsigned heads = __ballot_sync(0xffffffffu, head);
        if (head) {
            const unsigned later = heads & ~((2u << lane) - 1u);  // heads after this lane
            const uint32_t end = later ? (uint32_t)(__ffs(later) - 1) : (uint32_t)(32 - __clz(vm));
            atomicAdd(&s_hist[ps * kRadix + d], end - lane);
        }
    }
}

// Move-only ticks (several per launch, the state in registers between them): one
// entity per thread in 128-thread blocks, so a small entity count still spreads
// over many SMs (10,000 entities: 0.264 us per tick against 0.278 with the
// two-per-thread, 512-thread shape of k_step; equal at 200,000).
template <int RNG>
__global__ __launch_bounds__(kMoveThreads) void k_move(StepLaunch a) {
    chain_enter();
    const uint32_t stride = gridDim.x * kMoveThreads;
    for (uint32_t s = blockIdx.x * kMoveThreads + threadIdx.x; s < a.n; s += stride) {
        float2 p = a.st.pos[s];
        uint32_t h = a.st.head[s];
        const uint32_t h0 = h;
        const float sp = a.st.speed[s];
        uint4 r = make_uint4(0u, 0u, 0u, 0u);
        bool rl = false, rd = false;
        for (uint32_t t = 0; t < a.ticks; t++) step_entity<RNG>(a.map, a.dt, sp, p, h, r, rl, rd, a.st.rng + s, a.err);
        a.st.pos[s] = p;
        if (h != h0) a.st.head[s] = h;
        if (rd) a.st.rng[s] = r;
        if (a.rank_pos) {  // uniform: a tick that reuses the index
            const uint32_t q = a.rank[s];
            if (q < a.rank_n) a.rank_pos[q] = p;
        }
    }
}

// kStepPer entities per thread and iteration (slots s, s + stride, ...), their loads
// in flight before any is stepped.  One per thread at four 512-thread blocks per SM
// (32 registers): 0.122 ms at 16 M against 0.125 for two per thread at three blocks.
// DISP: the tick's largest displacement is measured too (StepLaunch::disp_max).
template <int RNG, bool KEY, bool DISP>
__global__ __launch_bounds__(kStepThreads, 4) void k_step(StepLaunch a) {
    __shared__ uint32_t s_hist[kMaxPasses * kRadix];
    __shared__ uint32_t s_morton[KEY ? 2048 : 1];
    __shared__ uint32_t s_disp;
    if (KEY) {  // shared memory only: overlaps the predecessor's tail
        for (uint32_t i = threadIdx.x; i < a.passes * kRadix; i += kStepThreads) s_hist[i] = 0u;
        for (uint32_t i = threadIdx.x; i < 2048u; i += kStepThreads) s_morton[i] = part1by1(i);
        if (DISP && threadIdx.x == 0) s_disp = 0u;
        __syncthreads();
    }
    chain_enter();
    uint32_t dbits = 0u;  // DISP: this thread's largest displacement (non-negative float bits order as floats)
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * kStepThreads;
    for (uint32_t i = blockIdx.x * kStepThreads + threadIdx.x; i < a.zero_a_words; i += stride) a.zero_a[i] = 0u;
    if (a.zero_b && blockIdx.x == 0 && threadIdx.x == 0) *a.zero_b = 0u;
    for (uint32_t base = blockIdx.x * kStepThreads; base < a.n; base += kStepPer * stride) {
        uint32_t sl[kStepPer];
        bool valid[kStepPer];
        float2 p[kStepPer];
        uint32_t h[kStepPer], h0[kStepPer];
        float sp[kStepPer];
#pragma unroll
        for (int u = 0; u < kStepPer; u++) {
            sl[u] = base + u * stride + threadIdx.x;
            valid[u] = sl[u] < a.n;
            p[u] = make_float2(0.f, 0.f);
            h[u] = h0[u] = 0u;
            sp[u] = 0.f;
            if (valid[u]) {
                p[u] = a.st.pos[sl[u]];
                if (a.ticks) {
                    h[u] = h0[u] = a.st.head[sl[u]];
                    sp[u] = a.st.speed[sl[u]];
                    if (DISP && a.first_bad && (h[u] & kHeadRoad) >= a.map.num_roads)
                        atomicMin(a.first_bad, a.id_base + sl[u]);
                }
            }
        }
        uint32_t key[kStepPer];
#pragma unroll
        for (int u = 0; u < kStepPer; u++) {
            key[u] = 0u;
            if (!valid[u]) continue;
            if (a.ticks) {
                uint4 r = make_uint4(0u, 0u, 0u, 0u);
                bool rl = false, rd = false;
                for (uint32_t t = 0; t < a.ticks; t++)
                    step_entity<RNG>(a.map, a.dt, sp[u], p[u], h[u], r, rl, rd, a.st.rng + sl[u], a.err);
                a.st.pos[sl[u]] = p[u];
                if (h[u] != h0[u]) {
                    a.st.head[sl[u]] = h[u];
                    if (a.host_head) a.host_head[a.id_base + sl[u]] = h[u];  // the caller's copy, by id
                }
                if (rd) {
                    a.st.rng[sl[u]] = r;
                    if (a.host_rng) a.host_rng[a.id_base + sl[u]] = r;
                }
            }
            if (KEY) {
                key[u] = tile_key(a.grid, p[u], s_morton);
                a.key[sl[u]] = key[u];
            }
        }
        if (KEY && a.hist) {
#pragma unroll
            for (int u = 0; u < kStepPer; u++) digit_counts<RNG, KEY>(key[u], valid[u], lane, a.passes, s_hist);
        }
        if (DISP) {
#pragma unroll
            for (int u = 0; u < kStepPer; u++) {
                if (!valid[u]) continue;
                const float2 o = a.index_pos[sl[u]];
                const float dx = fabsf(__fsub_rn(p[u].x, o.x)), dy = fabsf(__fsub_rn(p[u].y, o.y));
                const uint32_t b = dx <= 3.0e38f && dy <= 3.0e38f ? __float_as_uint(fmaxf(dx, dy)) : 0x7f800000u;
                dbits = b > dbits ? b : dbits;
            }
        }
    }
    if (DISP) {  // one global atomic per block (one per warp serialised on the word: 0.08 ms per 4 M)
        dbits = __reduce_max_sync(0xffffffffu, dbits);
        if (lane == 0 && dbits) atomicMax(&s_disp, dbits);
        __syncthreads();
        if (threadIdx.x == 0 && s_disp) atomicMax(a.disp_max, s_disp);
    }
    if (KEY && a.hist) {
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < a.passes * kRadix; i += kStepThreads) {
            const uint32_t c = s_hist[i];
            if (c) atomicAdd(&a.hist[i], c);
        }
    }
}

// One stable LSD radix pass over 8 bits of the key (Adinets & Merrill,
// "Onesweep", 2022).  Blocks take tiles in launch order through an atomic ticket,
// rank their ROWS x 256 items with warp-level multi-split (__match_any_sync) into
// per-warp digit counters, publish per-digit counts and resolve their global
// offsets by looking back over earlier tiles.  Every wait is bounded.  Tiles hold
// 4096 items, or 1024 when the count is known only on the device: those passes sort
// the few changed entries of an incremental update (about 230 K of 16 M), where a
// pass lasts about as long as one tile takes, so smaller tiles finish sooner
// (measured at 16 M: 15.7 us per pass against 22.9 with 4096).
//
// chain (pointers NULL: the caller clears the look-back words and the ticket):
// before its tiles, the pass zeroes the next pass's look-back words that their last
// use published (*next_dirty) and the next pass's ticket, and records in *my_dirty
// the words it publishes itself, so consecutive passes need no memset between them.
//
// Ranking runs in three sweeps over the rows so that no row waits for the
// previous one: (1) match every row's digits (group size, leader lane, rank inside
// the row); (2) each group's leader adds the group size to the warp's counter for
// its digit with an atomic that returns the previous count - a warp's shared-memory
// atomics take effect in issue order, i.e. in row order, which keeps the pass
// stable; (3) the previous counts are broadcast from the leaders (steps 2 and 3
// four rows at a time).  Values are read
// only for the local scatter, so they hold no registers during the ranking.
template <bool PERSIST, int ROWS>
__global__ __launch_bounds__(kSortThreads, 4) void k_onesweep(const uint32_t* __restrict__ keys_in,
                                                              const uint32_t* __restrict__ vals_in,
                                                              uint32_t* __restrict__ keys_out,
                                                              uint32_t* __restrict__ vals_out, uint32_t n,
                                                              uint32_t shift,
                                                              const uint32_t* __restrict__ digit_count,
                                                              uint32_t* lookback, uint32_t* ticket, uint32_t* err,
                                                              const uint32_t* __restrict__ n_dev, SweepChain chain,
                                                              uint32_t spin_limit) {
    constexpr int NW = kSortThreads / 32;
    constexpr uint32_t TILE = kSortThreads * ROWS;
    constexpr int G = ROWS < 4 ? ROWS : 4;  // rows whose counter atomics are in flight together
    static_assert(ROWS % G == 0, "whole groups of rows");
    static_assert(kSortThreads == (int)kRadix, "one thread per digit");
    constexpr uint32_t FULL = 0xffffffffu;
    __shared__ uint32_t s_keys[TILE];
    __shared__ uint32_t s_vals[TILE];
    __shared__ uint32_t s_whist[NW * kRadix];  // per-warp counts, then exclusive warp prefix
    __shared__ uint32_t s_local_start[kRadix];
    __shared__ uint32_t s_global_base[kRadix];
    __shared__ uint32_t s_warp[NW + 1];
    __shared__ uint32_t s_tile;

    const uint32_t tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    chain_enter();
    if (index_failed(err)) return;  // an earlier wait gave up: the input is incomplete
    if (n_dev) n = min(*n_dev, n);  // item count known only on the device (grid sized for n)
    const uint32_t tiles = n ? (n + TILE - 1u) / TILE : 1u;
    if (chain.next_lookback) {  // clear the next pass's look-back words and ticket
        const uint32_t words = *chain.next_dirty;
        for (uint32_t w = blockIdx.x * kSortThreads + tid; w < words; w += gridDim.x * kSortThreads)
            chain.next_lookback[w] = 0u;
        if (blockIdx.x == 0 && tid == 0) {
            *chain.next_ticket = 0u;
            *chain.my_dirty = tiles * kRadix;
        }
    }
    // this pass's digit offsets: the exclusive scan of its digit counts (thread d: digit d)
    const uint32_t digit_base = block_exclusive_scan<kSortThreads>(digit_count[tid], s_warp, nullptr);
  for (;;) {  // a block takes tiles until none is left (the grid may be smaller than the tiles)
    __syncthreads();  // the previous tile's shared memory is free
    if (tid == 0) s_tile = atomicAdd(ticket, 1u);
    for (uint32_t i = tid; i < NW * kRadix; i += kSortThreads) s_whist[i] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile;
    if (tile >= tiles) return;  // tiles past the end: no later tile waits for them
    const uint32_t base = tile * TILE;
    const uint32_t row0 = base + warp * (ROWS * 32) + lane;

    uint32_t k[ROWS], rk[ROWS];
#pragma unroll
    for (int r = 0; r < ROWS; r++) {
        const uint32_t idx = row0 + r * 32;
        k[r] = idx < n ? keys_in[idx] : 0u;
    }
    uint32_t* wh = s_whist + warp * kRadix;
    const uint32_t lt = lanemask_lt();
    // (1) per row: rank inside the row | leader lane << 8 | group size << 16
#pragma unroll
    for (int r = 0; r < ROWS; r++) {
        const uint32_t idx = row0 + r * 32;
        const bool ok = idx < n;
        const unsigned vm = __ballot_sync(FULL, ok);
        rk[r] = 0u;
        if (ok) {
            const unsigned peers = __match_any_sync(vm, (k[r] >> shift) & 0xffu);
            rk[r] = (uint32_t)__popc(peers & lt) | ((uint32_t)(__ffs(peers) - 1) << 8) |
                    ((uint32_t)__popc(peers) << 16);
        }
    }
    // (2) leaders take their group's counts, in row order, four rows in flight;
    // (3) broadcast from the leaders
#pragma unroll
    for (int r0 = 0; r0 < ROWS; r0 += G) {
        uint32_t old[G];
#pragma unroll
        for (int q = 0; q < G; q++) {
            const int r = r0 + q;
            old[q] = 0u;
            const uint32_t idx = row0 + r * 32;
            if (idx < n && ((rk[r] >> 8) & 0xffu) == lane)
                old[q] = atomicAdd(&wh[(k[r] >> shift) & 0xffu], rk[r] >> 16);
        }
#pragma unroll
        for (int q = 0; q < G; q++) {
            const int r = r0 + q;
            const uint32_t from_leader = __shfl_sync(FULL, old[q], (rk[r] >> 8) & 0x1fu);
            rk[r] = from_leader + (rk[r] & 0xffu);
        }
    }
    __syncthreads();

    // one thread per digit: warp prefix, block count, publication, look-back
    const uint32_t d = tid;
    uint32_t tot = 0u;
#pragma unroll
    for (int w = 0; w < NW; w++) {
        const uint32_t c = s_whist[w * kRadix + d];
        s_whist[w * kRadix + d] = tot;
        tot += c;
    }
    uint32_t* my_lb = lookback + (size_t)tile * kRadix + d;
    st_relaxed(my_lb, (tile == 0 ? kFlagPrefix : kFlagAgg) | tot);
    uint32_t excl = 0u;
    if (tile > 0) {
        // look back kLookBack tiles per round of loads
        int32_t j = (int32_t)tile - 1;
        uint32_t spins = 0u;
        bool done = false;
        while (!done) {
            uint32_t w[kLookBack];
#pragma unroll
            for (int q = 0; q < kLookBack; q++)
                w[q] = j - q >= 0 ? ld_relaxed(lookback + (size_t)(j - q) * kRadix + d) : kFlagPrefix;
            int take = kLookBack;  // predecessors consumed this round
            bool stop = false;
#pragma unroll
            for (int q = 0; q < kLookBack; q++) {
                if (stop) continue;
                if ((w[q] & kFlagMask) == 0u) {  // not published yet: poll it again
                    take = q;
                    stop = true;
                } else {
                    excl += w[q] & kValueMask;
                    if (w[q] & kFlagPrefix) {
                        done = true;
                        stop = true;
                    }
                }
            }
            if (done) break;
            j -= take;
            if (take < kLookBack) {
                if (++spins > spin_limit) {
                    atomicOr(err, kErrTimeout);
                    break;
                }
                __nanosleep(32);
            }
        }
        st_relaxed(my_lb, kFlagPrefix | ((excl + tot) & kValueMask));
    }
    s_global_base[d] = digit_base + excl;
    const uint32_t local_start = block_exclusive_scan<kSortThreads>(tot, s_warp, nullptr);
    s_local_start[d] = local_start;
    __syncthreads();  // every thread reads other digits' starts below

    // local scatter into shared memory (digit-major), then coalesced runs out
    uint32_t v[ROWS];
#pragma unroll
    for (int r = 0; r < ROWS; r++) {
        const uint32_t idx = row0 + r * 32;
        v[r] = idx < n ? (vals_in ? vals_in[idx] : idx) : 0u;
    }
#pragma unroll
    for (int r = 0; r < ROWS; r++) {
        const uint32_t idx = row0 + r * 32;
        if (idx < n) {
            const uint32_t dd = (k[r] >> shift) & 0xffu;
            const uint32_t lpos = s_local_start[dd] + s_whist[warp * kRadix + dd] + rk[r];
            if (lpos >= TILE) {  // unreachable: ranks and counts come from the same pass
                atomicOr(err, kErrOob);
                continue;
            }
            s_keys[lpos] = k[r];
            s_vals[lpos] = v[r];
        }
    }
    __syncthreads();
    const uint32_t count = (n - base) < TILE ? (n - base) : TILE;
#pragma unroll
    for (int r = 0; r < ROWS; r++) {  // independent rows: their shared loads overlap
        const uint32_t i = tid + r * kSortThreads;
        if (i >= count) continue;
        const uint32_t key = s_keys[i];
        const uint32_t dd = (key >> shift) & 0xffu;
        const uint32_t g = s_global_base[dd] + (i - s_local_start[dd]);
        if (g >= n) {  // only after a look-back that gave up; never write out of range
            atomicOr(err, kErrTimeout);
            continue;
        }
        keys_out[g] = key;
        vals_out[g] = s_vals[i];
    }
    if (!PERSIST) return;  // one tile per block
  }
}

// [start, end) of every occupied tile; the tile of a key is key >> ybits.
__global__ void k_ranges(const uint32_t* __restrict__ sk, uint32_t n, uint32_t* __restrict__ ranges,
                         uint32_t num_keys, uint32_t ybits) {
    // four consecutive sorted keys per thread (one 16-byte load when in range)
    const uint32_t p0 = (blockIdx.x * blockDim.x + threadIdx.x) * 4u;
    if (p0 >= n) return;
    uint32_t k[6];  // k[0] = key before p0, k[1..4] = keys p0..p0+3, k[5] = key after
    k[0] = p0 ? sk[p0 - 1] : 0xffffffffu;
    if (p0 + 4 <= n) {
        const uint4 v = *reinterpret_cast<const uint4*>(sk + p0);
        k[1] = v.x;
        k[2] = v.y;
        k[3] = v.z;
        k[4] = v.w;
        k[5] = p0 + 4 < n ? sk[p0 + 4] : 0xffffffffu;
    } else {
#pragma unroll
        for (int i = 1; i < 6; i++) k[i] = p0 + i - 1 < n ? sk[p0 + i - 1] : 0xffffffffu;
    }
#pragma unroll
    for (int i = 0; i < 6; i++) k[i] >>= ybits;  // tile codes (the sentinels stay above every tile)
#pragma unroll
    for (int i = 1; i <= 4; i++) {
        const uint32_t p = p0 + i - 1;
        if (p >= n || k[i] >= num_keys) continue;  // tiles are Morton codes of clamped tile coordinates
        if (k[i - 1] != k[i]) ranges[2ull * k[i]] = p;
        if (k[i + 1] != k[i]) ranges[2ull * k[i] + 1] = p + 1;
    }
}

// The query keeps the sorted positions of an entity's first kRegKeep neighbours in
// shared memory; entities with more take list_overflow, which walks their tiles again
// and holds up the whole warp.  At the 16 M workload 0.9 % of the entities have more
// than 4 neighbours (a quarter of the warps would wait) and 0.001 % more than 8.
constexpr int kRegKeep = 8;

// Exact ascending list of the cap smallest ids of one entity, written by
// insertion straight into its output slots; for the rare entities with more
// than kRegKeep neighbours.
__device__ __noinline__ void list_overflow(const uint32_t* __restrict__ sorted_slot,
                                           const float2* __restrict__ sorted_pos,
                                           const uint32_t* __restrict__ slot_id, const uint32_t* __restrict__ kstart,
                                           const TileGrid& g, uint32_t n, uint32_t p, uint32_t cap,
                                           uint32_t* out) {
    // the entity and its query box's tiles, read and recomputed here so the caller
    // keeps nothing live for them
    const float2 me = sorted_pos[p];
    const uint32_t x0 = tile_coord(__fsub_rn(me.x, g.reach), g.inv_cell, g.tiles_x);
    const uint32_t x1 = tile_coord(__fadd_rn(me.x, g.reach), g.inv_cell, g.tiles_x);
    const uint32_t y0 = tile_coord(__fsub_rn(me.y, g.reach), g.inv_cell, g.tiles_y);
    const uint32_t y1 = tile_coord(__fadd_rn(me.y, g.reach), g.inv_cell, g.tiles_y);
    uint32_t m = 0;
    for (uint32_t ty = y0; ty <= y1; ty++) {
        for (uint32_t tx = x0; tx <= x1; tx++) {
            const uint32_t t = morton2(tx, ty);
            const uint32_t q0 = kstart[t << g.ybits];
            const uint32_t q1 = kstart[(t + 1u) << g.ybits];
            const uint32_t qend = q1 < n ? q1 : n;
            for (uint32_t q = q0; q < qend; q++) {
                if (q == p || !in_range(sorted_pos[q], me, g.radius)) continue;
                const uint32_t s2 = sorted_slot[q];
                if (s2 >= n) continue;
                const uint32_t oid = slot_id ? slot_id[s2] : s2;
                if (m == cap && oid >= out[cap - 1]) continue;
                uint32_t j = m < cap ? m++ : cap - 1;
                while (j > 0 && out[j - 1] > oid) {
                    out[j] = out[j - 1];
                    j--;
                }
                out[j] = oid;
            }
        }
    }
}

#include "msim_query.cuh"
#include "msim_incsort.cuh"

__global__ void k_permute(const uint32_t* __restrict__ ss, EntityState src, EntityState dst, uint32_t n,
                          const uint32_t* err) {
    chain_enter();
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t s = !index_failed(err) && ss[p] < n ? ss[p] : p;
    dst.pos[p] = src.pos[s];
    dst.head[p] = src.head[s];
    dst.rng[p] = src.rng[s];
    dst.speed[p] = src.speed[s];
    dst.slot_id[p] = src.slot_id[s];
}

__global__ void k_export_state(EntityState st, uint32_t n, float2* pos, uint32_t* head, uint4* rng, float* speed) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t id = st.slot_id[s];
    if (id >= n) return;
    if (pos) pos[id] = st.pos[s];
    if (head) head[id] = st.head[s];
    if (rng) rng[id] = st.rng[s];
    if (speed) speed[id] = st.speed[s];
}

__global__ __launch_bounds__(kQueryThreads) void k_export_nbr(const uint32_t* sorted_slot, const uint32_t* slot_id,
                                                              const uint32_t* count, const uint32_t* list,
                                                              uint32_t n, uint32_t cap, uint32_t* out_count,
                                                              uint32_t* out_idx) {
    // the query's list layout: warp w's lists at w * 32 * cap, in lane order
    const uint32_t p = blockIdx.x * kQueryThreads + threadIdx.x;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t c = p < n ? count[p] : 0u;
    const uint32_t kept = c < cap ? c : cap;
    uint32_t incl = kept;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
    }
    if (p >= n) return;
    const uint32_t s = sorted_slot ? sorted_slot[p] : p;
    if (s >= n) return;
    const uint32_t id = slot_id ? slot_id[s] : s;  // NULL: slot s holds entity s
    if (id >= n) return;
    out_count[id] = c;
    if (out_idx && cap) {
        const uint32_t* src = list + (size_t)(p >> 5) * 32u * cap + (incl - kept);
        uint32_t* dst = out_idx + (size_t)id * cap;
        for (uint32_t j = 0; j < cap; j++) dst[j] = j < kept ? src[j] : 0xffffffffu;
    }
}

// Entity.hpp:33-46 record: color, randomState, pos, target, direction, roadIndex,
// initialized.  direction = update_direction(pos) (random_move.comp:830-839).
__global__ void k_export_aos(DeviceMap m, EntityState st, uint32_t n, float dt, uint4* out) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const uint32_t id = st.slot_id[s];
    if (id >= n) return;
    const float2 p = st.pos[s];
    const uint32_t h = st.head[s];
    const uint32_t road = h & kHeadRoad;
    float tx = p.x, ty = p.y, f = 1.f;
    if (road < m.num_roads) {
        const float4 rp = m.road_pos[road];
        tx = (h & kHeadToEnd) ? rp.z : rp.x;
        ty = (h & kHeadToEnd) ? rp.w : rp.y;
        if (m.factor) f = m.factor[road];
    }
    const float step = __fmul_rn(__fmul_rn(st.speed[s], f), dt);
    const float dx = __fsub_rn(tx, p.x), dy = __fsub_rn(ty, p.y);
    const float len = __fsqrt_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)));
    float dirx = 0.f, diry = 0.f;
    if (len != 0.f) {
        dirx = __fmul_rn(__fdiv_rn(dx, len), step);
        diry = __fmul_rn(__fdiv_rn(dy, len), step);
    }
    uint4* rec = out + (size_t)id * 4;
    rec[0] = make_uint4(__float_as_uint(1.f), 0u, 0u, __float_as_uint(1.f));  // red until a collision tick
    rec[1] = st.rng[s];
    rec[2] = make_uint4(__float_as_uint(p.x), __float_as_uint(p.y), __float_as_uint(tx), __float_as_uint(ty));
    rec[3] = make_uint4(__float_as_uint(dirx), __float_as_uint(diry), road, 1u);
}

// collision colours of the last neighbour tick (random_move.comp:545-549, 876)
__global__ void k_export_colors(const uint32_t* sorted_slot, const uint32_t* slot_id, const uint32_t* count,
                                 uint32_t n, uint4* out) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const uint32_t s = sorted_slot ? sorted_slot[p] : p;
    if (s >= n) return;
    const uint32_t id = slot_id[s];
    if (id >= n) return;
    const bool hit = count[p] > 0u;
    out[(size_t)id * 4] = make_uint4(0u, hit ? 0u : __float_as_uint(1.f), hit ? __float_as_uint(1.f) : 0u,
                                     __float_as_uint(1.f));
}

// First entity whose heading names a road >= num_roads (atomicMin into *first_bad).
__global__ void k_check_roads(const uint32_t* __restrict__ head, uint32_t n, uint32_t num_roads, uint32_t base,
                              uint32_t* first_bad) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool bad = i < n && (head[i] & kHeadRoad) >= num_roads;
    const unsigned m = __ballot_sync(0xffffffffu, bad);
    if (m && (threadIdx.x & 31) == (uint32_t)(__ffs(m) - 1)) atomicMin(first_bad, base + i);
}

__global__ void k_fill_f32(float* out, uint32_t n, float v) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = v;
}

// out[q] = pos[P[q]] where lo <= P[q] < lo + cnt (host tick, one uploaded chunk):
// kGatherPer rows of 256 consecutive q per thread and round, every slot load of a
// thread issued before its position loads.
constexpr uint32_t kGatherPer = 4;
__global__ __launch_bounds__(256) void k_gather_chunk(const uint32_t* __restrict__ P, uint32_t n, uint32_t lo,
                                                      uint32_t cnt, const float2* __restrict__ pos,
                                                      float2* __restrict__ out) {
    const uint32_t stride = gridDim.x * 256u * kGatherPer;
    for (uint32_t base = blockIdx.x * 256u * kGatherPer + threadIdx.x; base < n; base += stride) {
        uint32_t sl[kGatherPer];
#pragma unroll
        for (uint32_t k = 0; k < kGatherPer; k++) {
            const uint32_t q = base + k * 256u;
            sl[k] = q < n ? P[q] - lo : 0xffffffffu;  // chunk-relative slot (wraps below lo)
        }
#pragma unroll
        for (uint32_t k = 0; k < kGatherPer; k++)
            if (sl[k] < cnt) out[base + k * 256u] = pos[lo + sl[k]];
    }
}

__device__ __forceinline__ uint32_t abs_bits(float v) {  // |v| as ordered bits; NaN / inf: +inf
    const float a = fabsf(v);
    return a <= 3.0e38f ? __float_as_uint(a) : 0x7f800000u;
}

__global__ __launch_bounds__(256) void k_bounds(const float* __restrict__ speed, const float2* __restrict__ pos,
                                                uint32_t n, uint32_t* out) {
    __shared__ uint32_t s_max[2];
    if (threadIdx.x == 0) s_max[0] = s_max[1] = 0u;
    __syncthreads();
    uint32_t ms = 0u, mp = 0u;
    for (uint32_t i = blockIdx.x * 256u + threadIdx.x; i < n; i += gridDim.x * 256u) {
        const float2 p = pos[i];
        ms = max(ms, abs_bits(speed[i]));
        mp = max(mp, max(abs_bits(p.x), abs_bits(p.y)));
    }
    ms = __reduce_max_sync(0xffffffffu, ms);
    mp = __reduce_max_sync(0xffffffffu, mp);
    if ((threadIdx.x & 31u) == 0) {
        atomicMax(&s_max[0], ms);
        atomicMax(&s_max[1], mp);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicMax(&out[0], s_max[0]);
        atomicMax(&out[1], s_max[1]);
    }
}

__global__ void k_iota(uint32_t* out, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = i;
}

inline unsigned blocks_for(uint32_t n, unsigned threads) { return (unsigned)((n + threads - 1) / threads); }

// Launch of a chain kernel (see chain_enter).
template <typename... KArgs, typename... Args>
cudaError_t launch_chained(void (*kernel)(KArgs...), unsigned grid, unsigned block, cudaStream_t s, Args... args) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace


cudaError_t configure_kernels(uint32_t) { return cudaSuccess; }

int step_blocks_for(int device, uint32_t n) {
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_step<0, true, false>, kStepThreads, 0);
    if (sms <= 0) sms = 1;
    if (per_sm <= 0) per_sm = 1;
    long long want = (long long)sms * per_sm;
    long long need = (n + kStepThreads - 1) / kStepThreads;
    if (need < 1) need = 1;
    return (int)(want < need ? want : need);
}

cudaError_t launch_init_entities(cudaStream_t s, const DeviceMap& m, EntityState st, uint32_t n, uint32_t rng_kind,
                                 uint64_t seed, uint32_t placement, float smin, float smax) {
    if (n == 0) return cudaSuccess;
    unsigned blocks = blocks_for(n, 256);
    if (blocks > 65535u * 8u) blocks = 65535u * 8u;
    k_init<<<blocks, 256, 0, s>>>(m, st, n, rng_kind, seed, placement, smin, smax);
    return cudaGetLastError();
}

cudaError_t launch_step(cudaStream_t s, const StepLaunch& a) {
    if (a.n == 0) return cudaSuccess;
    const bool key = a.key != nullptr;
    if (a.rank_pos && (key || a.ticks != 1 || !a.rank)) return cudaErrorInvalidValue;
    if (!key && a.ticks > 0 && !a.host_head && !a.host_rng) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const unsigned blocks = std::min<unsigned>(blocks_for(a.n, kMoveThreads), 16u * (unsigned)std::max(sms, 1));
        return a.rng_kind == 1 ? launch_chained(k_move<1>, blocks, kMoveThreads, s, a)
                               : launch_chained(k_move<0>, blocks, kMoveThreads, s, a);
    }
    if (a.disp_max) {  // a host tick that queries the previous index (keys, one tick)
        if (!key || !a.index_pos || a.ticks != 1) return cudaErrorInvalidValue;
        return a.rng_kind == 1 ? launch_chained(k_step<1, true, true>, a.blocks, kStepThreads, s, a)
                               : launch_chained(k_step<0, true, true>, a.blocks, kStepThreads, s, a);
    }
    if (a.rng_kind == 1) {
        return key ? launch_chained(k_step<1, true, false>, a.blocks, kStepThreads, s, a)
                   : launch_chained(k_step<1, false, false>, a.blocks, kStepThreads, s, a);
    } else {
        return key ? launch_chained(k_step<0, true, false>, a.blocks, kStepThreads, s, a)
                   : launch_chained(k_step<0, false, false>, a.blocks, kStepThreads, s, a);
    }
    return cudaGetLastError();
}

cudaError_t launch_onesweep(cudaStream_t s, const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out,
                            uint32_t* vals_out, uint32_t n, uint32_t shift, const uint32_t* digit_count,
                            uint32_t* lookback, uint32_t* ticket, uint32_t* err, const uint32_t* n_dev,
                            const SweepChain* chain, uint32_t spin_limit) {
    if (n == 0) return cudaSuccess;
    static bool carveout = false;  // prefer the largest shared-memory carveout: 4 blocks of 43 KB per SM
    if (!carveout) {
        cudaFuncSetAttribute(k_onesweep<false, kSortRows>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        cudaFuncSetAttribute(k_onesweep<true, kSortRowsDev>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        cudaGetLastError();
        carveout = true;
    }
    const SweepChain ch = chain ? *chain : SweepChain{};
    if (n_dev) {  // count known on the device only: a resident grid that loops over tiles
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const unsigned grid =
            std::min<unsigned>(blocks_for(n, kSortThreads * kSortRowsDev), 4u * (unsigned)(sms > 0 ? sms : 1));
        return launch_chained(k_onesweep<true, kSortRowsDev>, grid, kSortThreads, s, keys_in, vals_in, keys_out,
                              vals_out, n, shift, digit_count, lookback, ticket, err, n_dev, ch, spin_limit);
    }
    return launch_chained(k_onesweep<false, kSortRows>, blocks_for(n, kSortTile), kSortThreads, s, keys_in, vals_in,
                          keys_out, vals_out, n, shift, digit_count, lookback, ticket, err, n_dev, ch, spin_limit);
}

size_t sort_lookback_words(uint32_t n) {
    const size_t tiles = std::max<size_t>((n + kSortTile - 1) / kSortTile,
                                          (n + kSortThreads * kSortRowsDev - 1) / (kSortThreads * kSortRowsDev));
    return std::max<size_t>(tiles, 1) * kRadix;
}

cudaError_t launch_ranges(cudaStream_t s, const uint32_t* sorted_key, uint32_t n, uint2* ranges, uint32_t num_keys,
                          uint32_t ybits) {
    if (n == 0) return cudaSuccess;
    k_ranges<<<blocks_for((n + 3) / 4, 256), 256, 0, s>>>(sorted_key, n, reinterpret_cast<uint32_t*>(ranges), num_keys,
                                                          ybits);
    return cudaGetLastError();
}

uint32_t kstart_chunks(uint64_t num_keys) { return kstart_chunk_cap(num_keys); }

cudaError_t launch_kstart(cudaStream_t s, const uint32_t* sorted_key, uint32_t n, uint32_t* kstart, uint32_t num_keys,
                          uint4* chunks, uint32_t* chunk_count, uint32_t* kernels, const uint32_t* sorted_slot,
                          const float2* pos, float2* sorted_pos, const uint32_t* err) {
    if (kernels) *kernels = 0;
    if (num_keys == 0) return cudaSuccess;
    if (kernels) *kernels = 1;
    const uint64_t entries = (uint64_t)num_keys + 1u;
    const bool gather = sorted_slot && pos && sorted_pos && n > 0;
    if ((uint64_t)n > 8u * entries) {  // many positions per key
        k_kstart_search<<<(unsigned)((entries + 255u) / 256u), 256, 0, s>>>(sorted_key, n, kstart, num_keys, err);
        if (gather) {
            k_gather_pos<<<blocks_for(n, 256), 256, 0, s>>>(sorted_slot, pos, n, sorted_pos, err);
            if (kernels) *kernels = 2;
        }
    } else if (chunks && chunk_count) {
        const uint32_t cap = kstart_chunk_cap(num_keys);
        cudaError_t e = cudaMemsetAsync(chunk_count, 0, sizeof(uint32_t), s);
        if (e != cudaSuccess) return e;
        e = launch_chained(k_kstart_pos, blocks_for(n + 1u, 256), 256, s, sorted_key, n, kstart, num_keys, chunks,
                           chunk_count, cap, sorted_slot, pos, sorted_pos, err);
        if (e != cudaSuccess) return e;
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        e = launch_chained(k_kstart_fill, 4u * (sms > 0 ? sms : 1), 256, s, chunks, chunk_count, cap, kstart, err);
        if (e != cudaSuccess) return e;
        if (kernels) *kernels = 2;
    } else {
        const uint64_t warps = (entries + kKstartWindow - 1u) / kKstartWindow;
        k_kstart<<<(unsigned)((warps + 7u) / 8u), 256, 0, s>>>(sorted_key, n, kstart, num_keys, err);
        if (gather) {
            k_gather_pos<<<blocks_for(n, 256), 256, 0, s>>>(sorted_slot, pos, n, sorted_pos, err);
            if (kernels) *kernels = 2;
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_query(cudaStream_t s, uint32_t cap, const uint32_t* kstart, const uint32_t* sorted_slot,
                         const float2* sorted_pos, const uint32_t* slot_id, TileGrid grid, uint32_t n, uint32_t* count,
                         uint32_t* list, unsigned long long* pair_bins, const uint32_t* err, uint32_t* count_by_id) {
    if (n == 0) return cudaSuccess;
    static bool carveout = false;  // 16 blocks of ~9.5 KB per SM
    if (!carveout) {
        cudaFuncSetAttribute(k_query<true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        cudaFuncSetAttribute(k_query<false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        cudaGetLastError();
        carveout = true;
    }
    if (cap > 0 && list)
        k_query<true><<<blocks_for(n, kQueryThreads), kQueryThreads, 0, s>>>(kstart, sorted_slot, sorted_pos, slot_id,
                                                                            grid, n, cap, count, list, pair_bins, err,
                                                                            count_by_id);
    else
        k_query<false><<<blocks_for(n, kQueryThreads), kQueryThreads, 0, s>>>(kstart, sorted_slot, sorted_pos, slot_id,
                                                                             grid, n, 0u, count, nullptr, pair_bins, err,
                                                                             count_by_id);
    return cudaGetLastError();
}

cudaError_t launch_check_roads(cudaStream_t s, const uint32_t* head, uint32_t n, uint32_t num_roads,
                               uint32_t* first_bad) {
    cudaError_t e = cudaMemsetAsync(first_bad, 0xff, sizeof(uint32_t), s);
    if (e != cudaSuccess) return e;
    return launch_check_roads_range(s, head, 0, n, num_roads, first_bad);
}

cudaError_t launch_check_roads_range(cudaStream_t s, const uint32_t* head, uint32_t first, uint32_t n,
                                     uint32_t num_roads, uint32_t* first_bad) {
    if (n == 0) return cudaSuccess;
    k_check_roads<<<blocks_for(n, 256), 256, 0, s>>>(head + first, n, num_roads, first, first_bad);
    return cudaGetLastError();
}

cudaError_t launch_fill(cudaStream_t s, float* out, uint32_t n, float v) {
    if (n == 0) return cudaSuccess;
    k_fill_f32<<<blocks_for(n, 256), 256, 0, s>>>(out, n, v);
    return cudaGetLastError();
}

uint32_t mark_tiles(uint32_t n) { return (n + kMarkTile - 1u) / kMarkTile; }
uint32_t merge_tiles(uint32_t n) { return (n + kMergeTile - 1u) / kMergeTile; }

cudaError_t launch_mark(cudaStream_t s, const uint32_t* P, bool identity, const uint32_t* PK, const uint32_t* NK,
                        uint32_t n, uint32_t passes, uint32_t* a_key, uint32_t* a_val, uint32_t* b_key,
                        uint32_t* b_val, uint32_t* hist, unsigned long long* lookback, uint32_t* ticket,
                        uint32_t* counts, uint32_t* err, unsigned long long* changed_total, uint32_t spin_limit) {
    if (n == 0) return cudaMemsetAsync(counts, 0, 2 * sizeof(uint32_t), s);
    const uint32_t tiles = mark_tiles(n);
    return launch_chained(k_mark, tiles, kMarkThreads, s, P, identity ? 1u : 0u, PK, NK, n, passes, a_key, a_val, b_key,
                          b_val, hist, lookback, ticket, tiles, counts, err, changed_total, spin_limit);
}

cudaError_t launch_merge(cudaStream_t s, const uint32_t* a_key, const uint32_t* a_val, const uint32_t* b_key,
                         const uint32_t* b_val, const uint32_t* counts, uint32_t* split, uint32_t n,
                         uint32_t* out_key, uint32_t* out_val, const float2* pos, float2* sorted_pos,
                         uint32_t* kstart, uint32_t num_keys, uint4* chunks, uint32_t* chunk_count, uint32_t* err,
                         uint32_t* kernels, bool chunk_count_zeroed, uint32_t* rank) {
    if (kernels) *kernels = 0;
    if (n == 0 || num_keys == 0) return cudaSuccess;
    const uint32_t tiles = merge_tiles(n);
    const uint32_t cap = kstart_chunk_cap(num_keys);
    cudaError_t e = cudaSuccess;
    if (!chunk_count_zeroed)  // first: the three kernels chain
        e = cudaMemsetAsync(chunk_count, 0, sizeof(uint32_t), s);
    if (e == cudaSuccess)  // a warp per tile boundary
        e = launch_chained(k_merge_path, (tiles + 1u + 7u) / 8u, 256, s, a_key, b_key, counts, n, tiles + 1u, split,
                           static_cast<const uint32_t*>(err));
    if (e == cudaSuccess)
        e = launch_chained(k_merge, tiles, kMergeThreads, s, a_key, a_val, b_key, b_val, counts, split, n, out_key,
                           out_val, pos, sorted_pos, kstart, num_keys, chunks, chunk_count, cap, err, rank);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    e = launch_chained(k_kstart_fill, 4u * (sms > 0 ? sms : 1), 256, s, chunks, chunk_count, cap, kstart,
                       static_cast<const uint32_t*>(err));
    if (e == cudaSuccess && kernels) *kernels = 3;
    return e;
}

cudaError_t launch_gather_chunk(cudaStream_t s, const uint32_t* P, uint32_t n, uint32_t lo, uint32_t cnt,
                                const float2* pos, float2* out) {
    if (n == 0 || cnt == 0) return cudaSuccess;
    if (cnt > n || lo > n - cnt) return cudaErrorInvalidValue;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned want = 8u * (unsigned)std::max(sms, 1);
    const unsigned blocks = std::min<unsigned>(want, blocks_for(n, 256u * kGatherPer));
    k_gather_chunk<<<blocks, 256, 0, s>>>(P, n, lo, cnt, pos, out);
    return cudaGetLastError();
}

cudaError_t launch_bounds(cudaStream_t s, const float* speed, const float2* pos, uint32_t n, uint32_t* out) {
    if (n == 0) return cudaSuccess;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned blocks = std::min<unsigned>(8u * (unsigned)std::max(sms, 1), blocks_for(n, 256u));
    k_bounds<<<blocks, 256, 0, s>>>(speed, pos, n, out);
    return cudaGetLastError();
}

cudaError_t launch_iota(cudaStream_t s, uint32_t* out, uint32_t n) {
    if (n == 0) return cudaSuccess;
    k_iota<<<blocks_for(n, 256), 256, 0, s>>>(out, n);
    return cudaGetLastError();
}

cudaError_t launch_permute(cudaStream_t s, const uint32_t* sorted_slot, EntityState src, EntityState dst, uint32_t n,
                           const uint32_t* err) {
    if (n == 0) return cudaSuccess;
    return launch_chained(k_permute, blocks_for(n, 256), 256, s, sorted_slot, src, dst, n, err);
}

cudaError_t launch_export_state(cudaStream_t s, EntityState st, uint32_t n, float2* pos, uint32_t* head, uint4* rng,
                                float* speed) {
    if (n == 0) return cudaSuccess;
    k_export_state<<<blocks_for(n, 256), 256, 0, s>>>(st, n, pos, head, rng, speed);
    return cudaGetLastError();
}

cudaError_t launch_export_neighbours(cudaStream_t s, const uint32_t* sorted_slot, const uint32_t* slot_id,
                                     const uint32_t* count, const uint32_t* list, uint32_t n, uint32_t cap,
                                     uint32_t* out_count, uint32_t* out_idx) {
    if (n == 0) return cudaSuccess;
    k_export_nbr<<<blocks_for(n, kQueryThreads), kQueryThreads, 0, s>>>(sorted_slot, slot_id, count, list, n, cap,
                                                                        out_count, out_idx);
    return cudaGetLastError();
}

cudaError_t launch_export_aos(cudaStream_t s, const DeviceMap& m, EntityState st, uint32_t n, float dt,
                              const uint32_t* sorted_slot, const uint32_t* count, void* out) {
    if (n == 0) return cudaSuccess;
    k_export_aos<<<blocks_for(n, 256), 256, 0, s>>>(m, st, n, dt, static_cast<uint4*>(out));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !count) return e;
    k_export_colors<<<blocks_for(n, 256), 256, 0, s>>>(sorted_slot, st.slot_id, count, n, static_cast<uint4*>(out));
    return cudaGetLastError();
}

}  // namespace msim
