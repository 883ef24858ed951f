// C ABI of the movement-sim per-tick path: context lifecycle, tick orchestration
// on the context's CUDA stream, exports back to the reference's layouts.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "msim_debug.h"
#include "msim_internal.h"
#include "msim_kernels.cuh"

namespace msim {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }
int fail(int code, const std::string& msg) {
    g_last_error = msg;
    return code;
}

// Device allocations left before an injected failure (msim_debug_fail_device_alloc);
// negative: no failure injected.
static std::atomic<long long> g_alloc_budget{-1};

bool device_malloc(void** p, size_t bytes) {
    *p = nullptr;
    long long b = g_alloc_budget.load();
    while (b >= 0) {
        if (b == 0) return false;  // injected: every allocation fails until reset
        if (g_alloc_budget.compare_exchange_weak(b, b - 1)) break;
    }
    if (cudaMalloc(p, bytes) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return false;
    }
    return true;
}

enum KernelId : uint32_t {
    K_INIT = 0,
    K_STEP,        // one tick + key + digit histogram (neighbour ticks)
    K_STEP_MULTI,  // several move-only ticks per launch
    K_SORT_PASS,
    K_KSTART,
    K_QUERY,
    K_PERMUTE,
    K_EXPORT,
    K_MARK,   // split of the previous order into unchanged / changed keys
    K_MERGE,  // merge + key-start table + sorted positions
    K_GATHER, // host tick: an uploaded chunk's positions into the previous sorted order
    K_MOVE,   // a tick that reuses the index: move + each position at its sorted position
    K_COUNT
};
static const char* const kKernelNames[K_COUNT] = {"k_init",   "k_step",   "k_step_multi", "k_onesweep",
                                                  "k_kstart", "k_query",  "k_permute",    "k_export",
                                                  "k_mark",   "k_merge",  "k_gather", "k_move"};

// msim_tick_host: at most this many chunks, each at least kHostChunkMin entities
constexpr uint32_t kHostChunks = 4;  // at 16 M: 4.09 ms per host tick; 8 chunks 4.16-4.18, 16 4.31
constexpr uint32_t kHostChunkMin = 65536;

}  // namespace msim

using namespace msim;

struct msim_ctx {
    int device = 0;
    uint32_t spin_limit = kDefaultSpinLimit;  // polls before a bounded device wait gives up
    uint32_t fault = 0, fault_arg = 0;        // injected fault (msim_debug_inject), one shot
    cudaStream_t stream = nullptr;
    msim_params params{};
    uint32_t n = 0, R = 0, C = 0;
    float world_w = 0.f, world_h = 0.f;
    // map
    float4* road_pos = nullptr;
    uint4* road_conn = nullptr;
    uint32_t* conn = nullptr;
    float* factor = nullptr;
    // entity state, double-buffered for re-ordering
    EntityState st[2]{};
    int cur = 0;
    // spatial index
    uint32_t* key = nullptr;
    uint32_t* sk[2] = {nullptr, nullptr};
    uint32_t* sv[2] = {nullptr, nullptr};
    uint32_t* hist = nullptr;
    uint32_t* lookback = nullptr;   // kMaxPasses regions of sort_region words, chained (see sweep_chain)
    uint32_t* tickets = nullptr;
    uint32_t* sort_dirty = nullptr; // per region: look-back words its last pass published
    bool chain_broken = false;      // a pass failed to launch: the regions' state is unknown
    size_t sort_region = 0;
    // The index the query reads (current buffer set).  Two sets, paired with the two
    // sorted-slot buffers: a tick's merge writes the set the previous tick's query does
    // not read, so that query overlaps the next tick up to its merge.
    uint32_t* kstart = nullptr;  // first sorted position of every key, 2^key_bits + 1 entries
    uint4* kstart_chunks = nullptr;  // long key gaps, filled by a second kernel
    float2* sorted_pos = nullptr;    // positions in sorted order (the query's candidates)
    uint32_t* kstart_chunk_count = nullptr;
    uint32_t* kstart_b[2] = {nullptr, nullptr};
    uint4* kstart_chunks_b[2] = {nullptr, nullptr};
    float2* sorted_pos_b[2] = {nullptr, nullptr};
    uint32_t* kstart_chunk_count_b[2] = {nullptr, nullptr};
    int ib = 0;  // current index buffer set
    size_t num_keys = 0;
    const uint32_t* sorted_key = nullptr;
    const uint32_t* sorted_slot = nullptr;
    bool have_sort = false;
    // incremental index update: the previous order split into unchanged (a) and
    // changed (b, sorted in place with ping-pong) keys, then merged
    bool order_identity = false;  // sorted_slot[q] == q (right after a re-ordering)
    bool chunk_count_zeroed = false;  // the move step of this tick zeroed the merge's long-gap counter
    bool slots_identity = false;  // slot s holds entity s (state set from the host, not re-ordered since)
    bool incremental = true;      // index updates from the previous order (else full sorts)
    uint32_t* a_key = nullptr;
    uint32_t* a_val = nullptr;
    uint32_t* b_key[2] = {nullptr, nullptr};
    uint32_t* b_val[2] = {nullptr, nullptr};
    uint32_t* ab_counts = nullptr;
    unsigned long long* mark_lookback = nullptr;
    uint32_t* mark_ticket = nullptr;
    size_t update_words = 0;  // hist, mark ticket and mark look-back lie together: one memset per update
    uint32_t* merge_split = nullptr;
    // entries that went through the radix passes since the stats were reset: full
    // sorts counted on the host, incremental updates' changed entries on the device
    unsigned long long* sorted_dev = nullptr;
    uint64_t sorted_host = 0;
    uint64_t index_updates = 0;
    // Index reuse: neighbour ticks between index updates query the last index with
    // every box widened by how far an entity can have moved since.  reuse_ticks = move
    // ticks since the keys of the current index were computed (-1: the index does not
    // describe the state); step_bound = bound on any entity's displacement in one tick,
    // per coordinate (valid with bounds_valid; from max |speed|, max |road factor|, dt
    // and the largest coordinate, for the rounding); reuse_pos = the positions of a
    // reusing tick in the index's sorted order, alternating between ticks.
    bool reuse = true;
    int64_t reuse_ticks = -1;
    bool bounds_valid = false;
    double step_bound = 0.0;
    double max_factor = 1.0;
    double maxc = 0.0;
    uint32_t* bounds_dev = nullptr;  // [max |speed|, max |coordinate|] as float bits
    float2* reuse_pos[2] = {nullptr, nullptr};
    // rank[slot] = sorted position of the slot in the current index, written by the
    // merge once allocated (rank_valid: it describes the current index); a reusing
    // tick's move then writes each position there itself (no gather pass)
    uint32_t* rank = nullptr;
    bool rank_valid = false;
    cudaEvent_t ev_reuse_read[2] = {nullptr, nullptr};
    bool reuse_read_pending[2] = {false, false};
    int reuse_buf = 0;
    // Host ticks: with the index built from the state they start from (reuse_ticks ==
    // 0, slot = id), the query reads it with boxes widened by the tick's measured
    // largest displacement (the skin query); skin_pos = the new positions in that
    // index's sorted order; disp = that displacement (device word, float bits);
    // disp_host = page-locked words: [0] its copy, [1] the device status as the query
    // left it.
    bool state_free_event = false;
    uint64_t host_ticks = 0, skin_queries = 0;  // since the stats were reset
    float last_disp = 0.f;  // ev_state_free marks the last read of the spare state buffer
    float2* skin_pos = nullptr;
    uint32_t* disp = nullptr;
    uint32_t* disp_host = nullptr;
    cudaEvent_t ev_disp = nullptr, ev_query = nullptr, ev_state_free = nullptr;
    // neighbours
    // query_slot: the sorted slots of the index the last query ran on (its counts and
    // lists are in that order; a host tick's background update moves sorted_slot on)
    const uint32_t* query_slot = nullptr;
    uint32_t* nbr_count = nullptr;
    uint32_t* nbr_list = nullptr;
    unsigned long long* pairs = nullptr;
    bool have_nbr = false;
    uint32_t* err = nullptr;
    uint32_t* check = nullptr;  // first invalid heading found by msim_set_entities
    TileGrid grid{};
    uint32_t passes = 1;
    uint32_t resort = 16;
    uint32_t since_permute = 0;
    int step_blocks = 1;
    uint64_t tick = 0;
    size_t device_bytes = 0;
    std::vector<void*> allocs;
    void* stage = nullptr;
    size_t stage_bytes = 0;
    // profiling
    bool profiling = false;
    uint64_t launch_count = 0;  // kernels launched since creation
    struct Pending {
        uint32_t kernel;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    std::vector<cudaEvent_t> pool;
    uint64_t launches[K_COUNT] = {};
    double ms[K_COUNT] = {};
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    bool timer_open = false;
    // per-tick phase events (msim_set_tick_timing): before the move, after it, after
    // the query; recorded on the stream that runs each phase, so the query keeps its
    // own stream
    bool tick_timing = false;
    bool tick_recorded = false;
    cudaEvent_t ev_tick[3] = {nullptr, nullptr, nullptr};
    // the query of tick t runs on qstream while the main stream moves tick t + 1
    cudaStream_t qstream = nullptr;
    cudaEvent_t ev_index = nullptr;  // key-start table and sorted positions of tick t ready
    cudaEvent_t ev_read[2] = {nullptr, nullptr};  // the last query on index buffer set b is done
    bool read_pending[2] = {false, false};
    // host round trip (msim_tick_host): upload and download streams, per-chunk events
    cudaStream_t up = nullptr, down = nullptr;
    cudaEvent_t ev_start = nullptr;
    cudaEvent_t ev_up[kHostChunks] = {};
    cudaEvent_t ev_moved[kHostChunks] = {};

    DeviceMap dmap() const {
        DeviceMap m;
        m.road_pos = road_pos;
        m.road_conn = road_conn;
        m.conn = conn;
        m.factor = factor;
        m.num_roads = R;
        m.num_conn = C;
        return m;
    }
};

namespace {

int cuda_fail(cudaError_t e, const char* what) {
    return fail(MSIM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(expr, what)                                   \
    do {                                                 \
        cudaError_t e_ = (expr);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)
// A launch of a tick's kernel under a Prof p: an injected fault (MSIM_FAULT_LAUNCH)
// reports a launch failure instead of issuing it.
#define CKL(p, expr, what) CK(inject_launch((p).c) ? cudaErrorLaunchFailure : (expr), what)

template <typename T>
int dalloc(msim_ctx* c, T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    void* raw = nullptr;
    if (!device_malloc(&raw, count * sizeof(T)))
        return fail(MSIM_ERR_NOMEM, "device allocation of " + std::to_string(count * sizeof(T)) + " bytes failed");
    c->allocs.push_back(raw);
    c->device_bytes += count * sizeof(T);
    *p = static_cast<T*>(raw);
    return MSIM_OK;
}

void free_all(msim_ctx* c) {
    for (void* p : c->allocs) cudaFree(p);
    c->allocs.clear();
    if (c->stage) cudaFree(c->stage);
    c->stage = nullptr;
    for (auto& pd : c->pending) {
        c->pool.push_back(pd.a);
        c->pool.push_back(pd.b);
    }
    c->pending.clear();
    for (cudaEvent_t e : c->pool) cudaEventDestroy(e);
    c->pool.clear();
    if (c->t0) cudaEventDestroy(c->t0);
    if (c->t1) cudaEventDestroy(c->t1);
    if (c->ev_index) cudaEventDestroy(c->ev_index);
    for (int k = 0; k < 3; k++)
        if (c->ev_tick[k]) cudaEventDestroy(c->ev_tick[k]);
    for (int b = 0; b < 2; b++)
        if (c->ev_read[b]) cudaEventDestroy(c->ev_read[b]);
    if (c->qstream) cudaStreamDestroy(c->qstream);
    if (c->ev_start) cudaEventDestroy(c->ev_start);
    for (uint32_t k = 0; k < kHostChunks; k++) {
        if (c->ev_up[k]) cudaEventDestroy(c->ev_up[k]);
        if (c->ev_moved[k]) cudaEventDestroy(c->ev_moved[k]);
    }
    for (cudaEvent_t e : {c->ev_disp, c->ev_query, c->ev_state_free, c->ev_reuse_read[0], c->ev_reuse_read[1]})
        if (e) cudaEventDestroy(e);
    if (c->disp_host) cudaFreeHost(c->disp_host);
    c->disp_host = nullptr;
    if (c->up) cudaStreamDestroy(c->up);
    if (c->down) cudaStreamDestroy(c->down);
    if (c->stream) cudaStreamDestroy(c->stream);
}

cudaEvent_t pool_event(msim_ctx* c) {
    if (!c->pool.empty()) {
        cudaEvent_t e = c->pool.back();
        c->pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}

// An injected launch failure (MSIM_FAULT_LAUNCH): true for the launch it names.
bool inject_launch(msim_ctx* c) {
    if (c->fault != MSIM_FAULT_LAUNCH) return false;
    if (c->fault_arg > 0) {
        c->fault_arg--;
        return false;
    }
    c->fault = 0;
    return true;
}

// Records an event pair around one launch when profiling is on.
struct Prof {
    msim_ctx* c;
    uint32_t k;
    cudaEvent_t a = nullptr;
    Prof(msim_ctx* ctx, uint32_t kernel) : c(ctx), k(kernel) {
        c->launch_count++;
        if (c->profiling) {
            a = pool_event(c);
            cudaEventRecord(a, c->stream);
        }
    }
    ~Prof() {
        if (a) {
            cudaEvent_t b = pool_event(c);
            cudaEventRecord(b, c->stream);
            c->pending.push_back({k, a, b});
        }
    }
};

int drain_profile(msim_ctx* c) {
    if (c->pending.empty()) return MSIM_OK;
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    for (auto& pd : c->pending) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, pd.a, pd.b);
        c->launches[pd.kernel]++;
        c->ms[pd.kernel] += ms;
        c->pool.push_back(pd.a);
        c->pool.push_back(pd.b);
    }
    c->pending.clear();
    return MSIM_OK;
}

int ensure_stage(msim_ctx* c, size_t bytes) {
    if (c->stage_bytes >= bytes) return MSIM_OK;
    if (c->stage) cudaFree(c->stage);
    c->stage = nullptr;
    c->stage_bytes = 0;
    if (!device_malloc(&c->stage, bytes))
        return fail(MSIM_ERR_NOMEM, "device allocation of export staging (" + std::to_string(bytes) + " bytes) failed");
    c->stage_bytes = bytes;
    return MSIM_OK;
}

EntityState& cur_state(msim_ctx* c) { return c->st[c->cur]; }

// Widened queries (index reuse on neighbour ticks, the skin query of host ticks) are
// allowed while the widening is at most this fraction of the reach.  At the 16 M
// workload a tick moves an entity at most 0.16 m against a reach of 2 m, and the
// query costs about the same at any widening up to 2 m (tiles of 25.6 m, bands of
// 6.4 m: 0.385-0.400 ms); per tick with reuse, measured at 16 M / 1 M: 0.25 of the
// reach 0.616 / 0.0521 ms, 0.5 0.573 / 0.0473, 1.0 0.555 / 0.0447, 1.5 0.569 /
// 0.0437, 2.0 0.558 / 0.0437, 3.0 0.568 / 0.0437.  At densities where a query meets
// 17 or 70 neighbours it costs the same at 0 and 1.0 (1.41 and 22.4 ms at 1 M).
constexpr float kWidenLimit = 1.0f;

// rank[slot] (written by every later merge once allocated): false when the allocation
// fails.
bool ensure_rank(msim_ctx* c) {
    if (c->rank) return true;
    void* raw = nullptr;
    if (!device_malloc(&raw, sizeof(uint32_t) * std::max<size_t>(c->n, 1))) return false;
    c->allocs.push_back(raw);
    c->device_bytes += sizeof(uint32_t) * std::max<size_t>(c->n, 1);
    c->rank = static_cast<uint32_t*>(raw);
    c->rank_valid = false;
    return true;
}

// Buffers of the skin query (allocated by the first host tick that can use it): false
// when an allocation fails, and the tick then takes the usual order.
bool ensure_skin(msim_ctx* c) {
    if (c->skin_pos && c->disp && c->disp_host) return true;
    if (!c->skin_pos) {
        void* raw = nullptr;
        if (!device_malloc(&raw, sizeof(float2) * std::max<size_t>(c->n, 1))) return false;
        c->allocs.push_back(raw);
        c->device_bytes += sizeof(float2) * std::max<size_t>(c->n, 1);
        c->skin_pos = static_cast<float2*>(raw);
    }
    if (!c->disp) {
        void* raw = nullptr;
        if (!device_malloc(&raw, sizeof(uint32_t))) return false;
        c->allocs.push_back(raw);
        c->device_bytes += sizeof(uint32_t);
        c->disp = static_cast<uint32_t*>(raw);
    }
    if (!c->disp_host) {
        void* h = nullptr;
        if (cudaMallocHost(&h, 2 * sizeof(uint32_t)) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        c->disp_host = static_cast<uint32_t*>(h);
    }
    return true;
}

// Buffers of index reuse on the device path (allocated by the first reusing tick):
// false when an allocation fails, and the ticks then update the index every time.
bool ensure_reuse(msim_ctx* c) {
    if (!ensure_rank(c)) return false;
    for (int b = 0; b < 2; b++) {
        if (!c->reuse_pos[b]) {
            void* raw = nullptr;
            if (!device_malloc(&raw, sizeof(float2) * std::max<size_t>(c->n, 1))) return false;
            c->allocs.push_back(raw);
            c->device_bytes += sizeof(float2) * std::max<size_t>(c->n, 1);
            c->reuse_pos[b] = static_cast<float2*>(raw);
        }
        if (!c->ev_reuse_read[b] && cudaEventCreateWithFlags(&c->ev_reuse_read[b], cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            c->ev_reuse_read[b] = nullptr;
            return false;
        }
    }
    return true;
}

// Widened reach for queries that read an index built `ticks` move ticks ago: reach +
// ticks * step_bound, rounded up to a float.
float widened_reach(const msim_ctx* c, double ticks) {
    const double r = (double)c->grid.reach + ticks * c->step_bound;
    float rf = (float)r;
    if ((double)rf < r) rf = std::nextafter(rf, INFINITY);
    return rf;
}

StepLaunch step_args(msim_ctx* c, uint32_t ticks, bool key) {
    StepLaunch a;
    a.map = c->dmap();
    a.st = cur_state(c);
    a.n = c->n;
    a.dt = c->params.dt;
    a.ticks = ticks;
    a.rng_kind = c->params.rng_kind;
    a.key = key ? c->key : nullptr;
    a.hist = c->hist;
    a.grid = c->grid;
    a.passes = c->passes;
    a.err = c->err;
    a.blocks = c->step_blocks;
    return a;
}

// Device address of page-locked host memory (registered or from cudaMallocHost), or
// nullptr for any other pointer.
void* mapped_host(const void* p) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// The main stream waits for the queries still running on qstream that read index
// buffer set b (wait_reads) or any set (join_query).
int wait_reads(msim_ctx* c, int b) {
    if (!c->read_pending[b]) return MSIM_OK;
    CK(cudaStreamWaitEvent(c->stream, c->ev_read[b], 0), "cudaStreamWaitEvent");
    c->read_pending[b] = false;
    return MSIM_OK;
}

int join_query(msim_ctx* c) {
    int rc = wait_reads(c, 0);
    return rc != MSIM_OK ? rc : wait_reads(c, 1);
}

// The next index is written to buffer set b (the set paired with its sorted slots).
void use_index_buffers(msim_ctx* c, int b) {
    c->ib = b;
    c->kstart = c->kstart_b[b];
    c->kstart_chunks = c->kstart_chunks_b[b];
    c->sorted_pos = c->sorted_pos_b[b];
    c->kstart_chunk_count = c->kstart_chunk_count_b[b];
}

// Radix passes over the look-back regions: with two or more passes each pass
// clears the next one's region and ticket (the regions start zeroed at creation),
// so no memset runs between them; a single pass clears its own before it runs.
SweepChain sweep_chain(msim_ctx* c, uint32_t ps) {
    SweepChain ch;
    const uint32_t nx = (ps + 1u) % c->passes;
    ch.next_lookback = c->lookback + nx * c->sort_region;
    ch.next_ticket = c->tickets + nx;
    ch.next_dirty = c->sort_dirty + nx;
    ch.my_dirty = c->sort_dirty + ps;
    return ch;
}

// Also after a pass failed to launch (a later pass then did not clear the region the
// next sort starts with): every region, ticket and extent is zeroed again.
int clear_unchained(msim_ctx* c) {
    if (c->passes >= 2 && !c->chain_broken) return MSIM_OK;
    const size_t words = c->chain_broken ? kMaxPasses * c->sort_region : c->sort_region;
    CK(cudaMemsetAsync(c->lookback, 0, sizeof(uint32_t) * words, c->stream), "memset lookback");
    CK(cudaMemsetAsync(c->tickets, 0, sizeof(uint32_t) * kMaxPasses, c->stream), "memset tickets");
    CK(cudaMemsetAsync(c->sort_dirty, 0, sizeof(uint32_t) * kMaxPasses, c->stream), "memset look-back extents");
    c->chain_broken = false;
    return MSIM_OK;
}

int sort_keys(msim_ctx* c);

// MSIM_FAULT_SORT_TILE: the look-back chain about to start (the ticket that hands out
// its tiles) begins at tile 1, so tile 0 is never processed and tile 1's bounded
// wait for it runs out.
int inject_sort_tile(msim_ctx* c, uint32_t* ticket) {
    if (c->fault != MSIM_FAULT_SORT_TILE) return MSIM_OK;
    c->fault = 0;
    static const uint32_t one = 1u;
    CK(cudaMemcpyAsync(ticket, &one, sizeof(one), cudaMemcpyHostToDevice, c->stream), "inject sort fault");
    return MSIM_OK;
}

// key + histogram (of the current positions, or after one move tick) + radix sort
int sort_entities(msim_ctx* c, uint32_t move_ticks) {
    CK(cudaMemsetAsync(c->hist, 0, sizeof(uint32_t) * kMaxPasses * kRadix, c->stream), "memset hist");
    {
        Prof p(c, K_STEP);
        CKL(p, launch_step(c->stream, step_args(c, move_ticks, true)), "k_step");
    }
    if (c->tick_timing && move_ticks) CK(cudaEventRecord(c->ev_tick[1], c->stream), "cudaEventRecord");
    return sort_keys(c);
}

// radix sort of (key, slot) for keys and digit counts already in c->key / c->hist
int sort_keys(msim_ctx* c) {
    int rc = clear_unchained(c);
    if (rc != MSIM_OK) return rc;
    rc = join_query(c);  // the passes rewrite the sorted slots the last query reads
    if (rc != MSIM_OK) return rc;
    if ((rc = inject_sort_tile(c, c->tickets)) != MSIM_OK) return rc;
    c->chain_broken = true;  // until every pass has launched
    for (uint32_t ps = 0; ps < c->passes; ps++) {
        const uint32_t* kin = ps == 0 ? c->key : c->sk[(ps - 1) & 1];
        const uint32_t* vin = ps == 0 ? nullptr : c->sv[(ps - 1) & 1];
        const SweepChain ch = sweep_chain(c, ps);
        Prof p(c, K_SORT_PASS);
        CKL(p, launch_onesweep(c->stream, kin, vin, c->sk[ps & 1], c->sv[ps & 1], c->n, 8u * ps,
                           c->hist + ps * kRadix, c->lookback + ps * c->sort_region, c->tickets + ps, c->err,
                           nullptr, c->passes >= 2 ? &ch : nullptr, c->spin_limit),
           "k_onesweep");
    }
    c->chain_broken = false;
    c->sorted_key = c->sk[(c->passes - 1) & 1];
    c->sorted_slot = c->sv[(c->passes - 1) & 1];
    c->rank_valid = false;  // a full sort writes no ranks
    c->have_sort = true;
    c->sorted_host += c->n;
    c->index_updates++;
    return MSIM_OK;
}

int permute_state(msim_ctx* c) {
    // the target state buffer holds the slot ids a query two ticks back may still read
    int rc = join_query(c);
    if (rc != MSIM_OK) return rc;
    Prof p(c, K_PERMUTE);
    CKL(p, launch_permute(c->stream, c->sorted_slot, c->st[c->cur], c->st[1 - c->cur], c->n, c->err), "k_permute");
    c->cur = 1 - c->cur;
    c->have_sort = false;
    c->order_identity = true;  // slot q now holds the entity at sorted position q
    c->slots_identity = false;
    c->rank_valid = false;
    c->since_permute = 0;
    return MSIM_OK;
}

// Forget the index (new entity state in slot = id order): the next neighbour tick
// runs a full sort, and the one after re-orders the state by it.
void reset_index(msim_ctx* c) {
    c->reuse_ticks = -1;
    c->rank_valid = false;
    c->state_free_event = false;
    c->have_nbr = false;
    c->have_sort = false;
    c->sorted_key = nullptr;
    c->sorted_slot = nullptr;
    c->order_identity = false;
    c->since_permute = c->resort;
}

// tick-0 index: the reference's first dispatch only inserts every entity into its
// tree (random_move.comp:863-867); here: sort by tile and re-order the state.
int build_index(msim_ctx* c) {
    c->have_nbr = false;
    c->reuse_ticks = -1;
    c->bounds_valid = false;
    c->state_free_event = false;
    if (c->n == 0) return MSIM_OK;
    int rc = sort_entities(c, 0);
    if (rc != MSIM_OK) return rc;
    return permute_state(c);
}

// One tick of the move plus the index, from the previous sorted order: split it by
// whether each key changed, sort the changed entries, merge (writing the key-start
// table and the sorted positions on the way).  The update's scratch (digit counts,
// split ticket and look-back words) is cleared first, in one memset, before the
// move, so that the move step and the split run back to back.
int incremental_update(msim_ctx* c, bool positions = true, bool ranks = true);

int clear_update_scratch(msim_ctx* c) {
    CK(cudaMemsetAsync(c->hist, 0, sizeof(uint32_t) * c->update_words, c->stream), "memset update scratch");
    return MSIM_OK;
}

int incremental_index(msim_ctx* c) {
    c->chunk_count_zeroed = false;
    {
        Prof p(c, K_STEP);
        StepLaunch a = step_args(c, 1, true);
        a.hist = nullptr;  // the changed keys' digits are counted by k_mark
        // the move step clears the update's scratch and the long-gap counter of the index
        // set the merge will write (no memsets between the chained launches)
        a.zero_a = c->hist;
        a.zero_a_words = (uint32_t)c->update_words;
        a.zero_b = c->kstart_chunk_count_b[c->sorted_key == c->sk[0] ? 1 : 0];
        CKL(p, launch_step(c->stream, a), "k_step");
        c->chunk_count_zeroed = true;
    }
    if (c->tick_timing) CK(cudaEventRecord(c->ev_tick[1], c->stream), "cudaEventRecord");
    return incremental_update(c);
}

// The update itself, for new keys (by slot) already in c->key.  positions = false:
// the sorted positions are not written (a host tick whose next query reads the
// positions it gathers itself).  ranks = false: no ranks either (a host tick's slots
// are entity ids, in no spatial order: writing rank[slot] scatters at random, 0.12 ms
// more per update at 16 M, and moves placing positions by them cost 0.11 ms more per
// 4 M chunk than the gather passes).
int incremental_update(msim_ctx* c, bool positions, bool ranks) {
    NvtxRange range("msim index update");
    int rc = inject_sort_tile(c, c->mark_ticket);
    if (rc != MSIM_OK) return rc;
    {
        Prof p(c, K_MARK);
        CKL(p, launch_mark(c->stream, c->sorted_slot, c->order_identity, c->sorted_key, c->key, c->n, c->passes,
                       c->a_key, c->a_val, c->b_key[0], c->b_val[0], c->hist, c->mark_lookback, c->mark_ticket,
                       c->ab_counts, c->err, c->sorted_dev, c->spin_limit),
           "k_mark");
        c->index_updates++;
    }
    rc = clear_unchained(c);
    if (rc != MSIM_OK) return rc;
    c->chain_broken = true;  // until every pass has launched
    for (uint32_t ps = 0; ps < c->passes; ps++) {  // stable radix sort of the changed entries
        const SweepChain ch = sweep_chain(c, ps);
        Prof p(c, K_SORT_PASS);
        CKL(p, launch_onesweep(c->stream, c->b_key[ps & 1], c->b_val[ps & 1], c->b_key[(ps + 1) & 1],
                           c->b_val[(ps + 1) & 1], c->n, 8u * ps, c->hist + ps * kRadix,
                           c->lookback + ps * c->sort_region, c->tickets + ps, c->err, c->ab_counts + 1,
                           c->passes >= 2 ? &ch : nullptr, c->spin_limit),
           "k_onesweep");
    }
    c->chain_broken = false;
    // The merge writes the sorted slots and index buffer set the previous tick's query
    // does not read (that query may still run); it waits for the query before that.
    const int out = c->sorted_key == c->sk[0] ? 1 : 0;
    rc = wait_reads(c, out);
    if (rc != MSIM_OK) return rc;
    use_index_buffers(c, out);
    {
        Prof p(c, K_MERGE);
        uint32_t launched = 0;
        CKL(p, launch_merge(c->stream, c->a_key, c->a_val, c->b_key[c->passes & 1], c->b_val[c->passes & 1],
                        c->ab_counts, c->merge_split, c->n, c->sk[out], c->sv[out],
                        positions ? cur_state(c).pos : nullptr, positions ? c->sorted_pos : nullptr,
                        c->kstart, (uint32_t)c->num_keys, c->kstart_chunks, c->kstart_chunk_count, c->err,
                        &launched, c->chunk_count_zeroed, ranks ? c->rank : nullptr),
           "k_merge");
        c->rank_valid = ranks && c->rank != nullptr;
        c->chunk_count_zeroed = false;
        if (launched > 1) c->launch_count += launched - 1;
    }
    c->sorted_key = c->sk[out];
    c->sorted_slot = c->sv[out];
    c->order_identity = false;
    c->have_sort = true;
    return MSIM_OK;
}

int key_start_table(msim_ctx* c);
int run_query(msim_ctx* c, bool overlap, uint32_t* count_by_id = nullptr, const float2* pos = nullptr,
              const TileGrid* grid = nullptr);

// Bound on any entity's displacement in one move tick, per coordinate, for index
// reuse.  A move advances at most step = |speed| * |road factor| * dt toward its target
// and snaps to it when closer (the rest of the step is discarded), so it moves at most
// step; each coordinate's rounding adds at most half an ulp of the largest coordinate,
// which no later position exceeds (every move heads for a road end, so positions stay
// within max(largest coordinate now, largest map coordinate)).  Computed from the
// current state (one reduction and a read-back) while the index describes it
// (reuse_ticks == 0), so the bound covers every tick since the build.
int ensure_bounds(msim_ctx* c) {
    if (c->bounds_valid) return MSIM_OK;
    CK(cudaMemsetAsync(c->bounds_dev, 0, 2 * sizeof(uint32_t), c->stream), "memset bounds");
    CK(launch_bounds(c->stream, cur_state(c).speed, cur_state(c).pos, c->n, c->bounds_dev), "k_bounds");
    uint32_t h[2] = {0u, 0u};
    CK(cudaMemcpyAsync(h, c->bounds_dev, sizeof(h), cudaMemcpyDeviceToHost, c->stream), "read bounds");
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    float vmax = 0.f, cmax = 0.f;
    std::memcpy(&vmax, &h[0], sizeof(float));
    std::memcpy(&cmax, &h[1], sizeof(float));
    const double step = (double)vmax * c->max_factor * (double)c->params.dt * (1.0 + 0x1p-20) +
                        std::max((double)cmax, c->maxc) * 0x1p-22 + 1e-30;
    c->step_bound = std::isfinite(step) ? step : INFINITY;
    c->bounds_valid = true;
    return MSIM_OK;
}

int neighbour_tick(msim_ctx* c) {
    NvtxRange range("msim neighbour tick");
    int rc;
    if (c->tick_timing) CK(cudaEventRecord(c->ev_tick[0], c->stream), "cudaEventRecord");
    // Index reuse: while the widening of this tick's boxes stays within kWidenLimit of
    // the reach, the tick moves the entities (each position also written at its sorted
    // position in the index, by the ranks of the last update, or gathered there after
    // a full sort) and queries the index built reuse_ticks + 1 ticks before; the
    // widening costs about 10 % of the query over a reuse window at 16 M (0.40 ms
    // against 0.36-0.39), the update it skips (split, passes, merge) about 0.30 ms.
    const double ticks = c->reuse_ticks >= 0 ? (double)c->reuse_ticks + 1.0 : 0.0;
    bool reuse = false;
    if (c->reuse && c->sorted_key && !c->order_identity && c->reuse_ticks >= 0 && c->grid.reach > 0.f &&
        (c->bounds_valid || c->reuse_ticks == 0)) {
        if ((rc = ensure_bounds(c)) != MSIM_OK) return rc;
        reuse = ticks * c->step_bound <= (double)kWidenLimit * (double)c->grid.reach && ensure_reuse(c);
    }
    if (!reuse) {
        if (c->have_sort && c->since_permute >= c->resort) {
            rc = permute_state(c);
            if (rc != MSIM_OK) return rc;
        }
        if (c->reuse) ensure_reuse(c);  // so this update writes the ranks the next ticks use
        if (c->sorted_key && c->incremental) {
            rc = incremental_index(c);
            if (rc != MSIM_OK) return rc;
        } else {
            rc = sort_entities(c, 1);
            if (rc != MSIM_OK) return rc;
            rc = key_start_table(c);
            if (rc != MSIM_OK) return rc;
        }
        rc = run_query(c, true);
        if (rc == MSIM_OK) c->reuse_ticks = 0;
        return rc;
    }
    // the buffer the query two ticks back read (it may still run on the query stream)
    const int x = c->reuse_buf = 1 - c->reuse_buf;
    if (c->reuse_read_pending[x]) {
        CK(cudaStreamWaitEvent(c->stream, c->ev_reuse_read[x], 0), "cudaStreamWaitEvent");
        c->reuse_read_pending[x] = false;
    }
    {  // the move writes each position at its sorted position too, when the ranks are known
        Prof p(c, K_MOVE);
        StepLaunch a = step_args(c, 1, false);
        if (c->rank_valid) {
            a.rank = c->rank;
            a.rank_pos = c->reuse_pos[x];
            a.rank_n = c->n;
        }
        CKL(p, launch_step(c->stream, a), "k_step");
    }
    if (c->tick_timing) CK(cudaEventRecord(c->ev_tick[1], c->stream), "cudaEventRecord");
    if (!c->rank_valid) {
        Prof p(c, K_GATHER);
        CKL(p, launch_gather_chunk(c->stream, c->sorted_slot, c->n, 0, c->n, cur_state(c).pos, c->reuse_pos[x]),
            "k_gather_chunk");
    }
    TileGrid g = c->grid;
    g.reach = widened_reach(c, ticks);
    rc = run_query(c, true, nullptr, c->reuse_pos[x], &g);
    if (rc != MSIM_OK) return rc;
    if (!c->profiling) {  // the query ran on the query stream (see run_query)
        CK(cudaEventRecord(c->ev_reuse_read[x], c->qstream), "cudaEventRecord");
        c->reuse_read_pending[x] = true;
    }
    c->reuse_ticks = (int64_t)ticks;
    return MSIM_OK;
}

// key-start table and positions in sorted order, after a full sort
int key_start_table(msim_ctx* c) {
    c->order_identity = false;
    // after a full sort (every query joined): the set paired with the final slot buffer
    use_index_buffers(c, c->sorted_slot == c->sv[0] ? 0 : 1);
    Prof p(c, K_KSTART);
    uint32_t launched = 0;
    CKL(p, launch_kstart(c->stream, c->sorted_key, c->n, c->kstart, (uint32_t)c->num_keys, c->kstart_chunks,
                     c->kstart_chunk_count, &launched, c->sorted_slot, cur_state(c).pos, c->sorted_pos, c->err),
       "k_kstart");
    if (launched > 1) c->launch_count += launched - 1;
    return MSIM_OK;
}

// The radius query over the index just built.
// count_by_id (only with slots holding their own entity): the counts also by id.
// pos / grid (may be NULL): the positions in sorted order and the grid (its reach)
// instead of the index's own (the skin query of a host tick).
int run_query(msim_ctx* c, bool overlap, uint32_t* count_by_id, const float2* pos, const TileGrid* grid) {
    NvtxRange range("msim query");
    // The query reads only the index (key-start table, sorted slots and positions)
    // and slot ids: the next tick's move step may overwrite positions meanwhile.  With
    // profiling on everything stays on one stream so the kernel times do not overlap.
    cudaStream_t qs = c->stream;
    if (overlap && !c->profiling) {
        CK(cudaEventRecord(c->ev_index, c->stream), "cudaEventRecord");
        CK(cudaStreamWaitEvent(c->qstream, c->ev_index, 0), "cudaStreamWaitEvent");
        qs = c->qstream;
    }
    CK(cudaMemsetAsync(c->pairs, 0, sizeof(unsigned long long) * kPairBins, qs), "memset pairs");
    {
        Prof p(c, K_QUERY);
        // slots that hold their own entity need no id lookup
        CKL(p, launch_query(qs, c->params.cap, c->kstart, c->sorted_slot, pos ? pos : c->sorted_pos,
                        c->slots_identity ? nullptr : cur_state(c).slot_id, grid ? *grid : c->grid,
                        c->n, c->nbr_count, c->nbr_list, c->pairs, c->err,
                        c->slots_identity ? count_by_id : nullptr),
           "k_query");
    }
    if (qs != c->stream) {
        CK(cudaEventRecord(c->ev_read[c->ib], qs), "cudaEventRecord");
        c->read_pending[c->ib] = true;
    }
    if (c->tick_timing) {
        CK(cudaEventRecord(c->ev_tick[2], qs), "cudaEventRecord");
        c->tick_recorded = true;
    }
    c->query_slot = c->sorted_slot;
    c->have_nbr = true;
    c->since_permute++;
    return MSIM_OK;
}

int check_ctx(msim_ctx* c) {
    if (!c) return fail(MSIM_ERR_INVALID, "context is NULL");
    cudaError_t e = cudaSetDevice(c->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return MSIM_OK;
}

int sync_and_check(msim_ctx* c) {
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    uint32_t h = 0;
    CK(cudaMemcpy(&h, c->err, sizeof(h), cudaMemcpyDeviceToHost), "read device status");
    if (h) {
        CK(cudaMemsetAsync(c->err, 0, sizeof(uint32_t), c->stream), "clear device status");
        if (h & kErrTimeout) {
            // The kernels that read the index skipped their work after the wait gave
            // up, so the entity state is intact; the index is rebuilt from scratch (full
            // sort, every look-back region zeroed again) by the next neighbour tick.
            c->chain_broken = true;
            reset_index(c);
            return fail(MSIM_ERR_TIMEOUT, "a bounded device wait (index look-back) gave up; the neighbour results "
                                          "since the last successful sync are invalid, the entity state is kept");
        }
        return fail(MSIM_ERR_OOB, "a device-side index check failed (road or connection index out of range)");
    }
    return MSIM_OK;
}

}  // namespace

extern "C" {

const char* msim_last_error(void) { return g_last_error.c_str(); }
const char* msim_version(void) { return "msim-gb300 0.1 (sm_103a)"; }

uint32_t msim_kernel_count(void) { return K_COUNT; }
const char* msim_kernel_name(uint32_t k) { return k < K_COUNT ? kKernelNames[k] : ""; }

int msim_create(const msim_map* map, const msim_params* params, msim_ctx** out) {
    if (!out) return fail(MSIM_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!map || !params) return fail(MSIM_ERR_INVALID, "map or params is NULL");
    int rc = validate_map(*map);
    if (rc != MSIM_OK) return rc;
    const msim_params& p = *params;
    if (p.num_entities >= (1u << 30)) return fail(MSIM_ERR_INVALID, "num_entities must be < 2^30");
    if (p.rng_kind > 1) return fail(MSIM_ERR_INVALID, "unknown rng_kind");
    if (!std::isfinite(p.dt) || !(p.dt > 0.f)) return fail(MSIM_ERR_INVALID, "dt must be positive and finite");
    if (!std::isfinite(p.radius) || p.radius < 0.f) return fail(MSIM_ERR_INVALID, "radius must be finite and >= 0");
    if (p.cap > kMaxCap) return fail(MSIM_ERR_INVALID, "cap must be <= " + std::to_string(kMaxCap));
    if (p.cell_size < 0.f || !std::isfinite(p.cell_size)) return fail(MSIM_ERR_INVALID, "cell_size must be >= 0");
    if (p.flags & ~(MSIM_PARAM_FULL_SORT | MSIM_PARAM_INCREMENTAL | MSIM_PARAM_NO_REUSE))
        return fail(MSIM_ERR_INVALID, "unknown params flags");
    if ((p.flags & MSIM_PARAM_FULL_SORT) && (p.flags & MSIM_PARAM_INCREMENTAL))
        return fail(MSIM_ERR_INVALID, "MSIM_PARAM_FULL_SORT and MSIM_PARAM_INCREMENTAL exclude each other");

    msim_ctx* c = new (std::nothrow) msim_ctx();
    if (!c) return fail(MSIM_ERR_NOMEM, "out of host memory");
    cudaError_t e = cudaGetDevice(&c->device);
    if (e != cudaSuccess) {
        delete c;
        return cuda_fail(e, "cudaGetDevice");
    }
    c->params = p;
    // the incremental index update is the faster one at every size measured (62.5 K,
    // 250 K, 1 M and 16 M entities at the lattice density: 0.051 against 0.060 ms per
    // tick at 62.5 K, 0.092 against 0.114 at 1 M)
    c->incremental = (p.flags & MSIM_PARAM_FULL_SORT) == 0;
    c->reuse = (p.flags & MSIM_PARAM_NO_REUSE) == 0;
    c->n = p.num_entities;
    c->R = map->num_roads;
    c->C = map->num_connections;
    c->world_w = map->width;
    c->world_h = map->height;

    auto bail = [&](int code) {
        free_all(c);
        delete c;
        return code;
    };
    e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->qstream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
    if (cudaEventCreate(&c->t0) != cudaSuccess || cudaEventCreate(&c->t1) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_index, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_read[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_read[1], cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(MSIM_ERR_CUDA, "cudaEventCreate failed"));

    // ---- spatial grid ----
    double maxc = std::max((double)c->world_w, (double)c->world_h);
    for (uint64_t i = 0; i < 4ull * c->R; i++) maxc = std::max(maxc, std::fabs((double)map->road_pos[i]));
    const double radius = p.radius;
    // reach covers the rounding of |dx| in the predicate and of pos -/+ reach
    const double reach = radius * (1.0 + 0x1p-20) + maxc * 0x1p-20 + 1e-30;
    c->maxc = maxc;
    double cell = p.cell_size;
    if (cell <= 0.0) {
        // about four entities per tile at uniform density (entities on roads bunch up
        // more); with the bands below, the 24-bit key budget gives the fewest
        // candidates per query around this size on lattice road networks
        double area = (double)c->world_w * (double)c->world_h;
        cell = std::max(2.0 * reach, 2.0 * std::sqrt(area / std::max<double>(c->n, 1.0)));
    }
    cell = std::max(cell, 1e-3);
    uint32_t bits = 1;
    for (;;) {
        double tx = std::ceil((double)c->world_w / cell), ty = std::ceil((double)c->world_h / cell);
        tx = std::max(tx, 1.0);
        ty = std::max(ty, 1.0);
        double tmax = std::max(tx, ty);
        bits = 1;
        while ((double)(1u << bits) < tmax) bits++;
        if (bits <= 11) {
            c->grid.tiles_x = (uint32_t)tx;
            c->grid.tiles_y = (uint32_t)ty;
            break;
        }
        cell = std::max((double)c->world_w, (double)c->world_h) / 2048.0 * (1.0 + 1e-6);
    }
    c->grid.inv_cell = (float)(1.0 / cell);
    c->grid.bits = bits;
    c->grid.reach = (float)reach;
    c->grid.radius = p.radius;
    c->grid.d2_limit = sqrt_limit(p.radius);
    // y bands inside a tile fill the key up to 24 bits (3 radix passes), at most 64
    // bands, and keep the key-start table within about four entries per entity
    uint32_t nbits = 0;
    while (nbits < 31u && (1ull << (nbits + 1)) <= 4ull * std::max<uint64_t>(c->n, 1)) nbits++;
    const uint32_t budget = nbits > 2u * bits ? nbits - 2u * bits : 0u;
    c->grid.ybits = std::min<uint32_t>(std::min<uint32_t>(6u, 24u - 2u * bits), budget);
    c->grid.ybands = (float)(1u << c->grid.ybits);
    c->passes = (2 * bits + c->grid.ybits + 7) / 8;
    c->num_keys = (size_t)1 << (2 * bits + c->grid.ybits);
    // entities move a small fraction of a tile per tick, so the slot order stays close
    // to the sorted order for many ticks: measured at 16 M over 1000 ticks, 0.917 ms
    // per tick re-ordering every 16 ticks, 0.895 every 64, 0.894 every 128 (the other
    // kernels' times unchanged)
    c->resort = p.resort_interval ? p.resort_interval : 64u;
    c->sort_region = sort_lookback_words(c->n);

    // ---- device buffers ----
    const size_t n = c->n;
    if ((rc = dalloc(c, &c->road_pos, c->R)) || (rc = dalloc(c, &c->road_conn, c->R)) ||
        (rc = dalloc(c, &c->conn, (size_t)c->C + 1)))
        return bail(rc);
    for (int b = 0; b < 2; b++) {
        if ((rc = dalloc(c, &c->st[b].pos, n)) || (rc = dalloc(c, &c->st[b].head, n)) ||
            (rc = dalloc(c, &c->st[b].rng, n)) || (rc = dalloc(c, &c->st[b].speed, n)) ||
            (rc = dalloc(c, &c->st[b].slot_id, n)) || (rc = dalloc(c, &c->sk[b], n)) || (rc = dalloc(c, &c->sv[b], n)))
            return bail(rc);
    }
    // [digit counts | split ticket, pad | split look-back words (8-byte aligned)]
    c->update_words = (size_t)kMaxPasses * kRadix + 2u + 2u * (size_t)mark_tiles(c->n);
    if ((rc = dalloc(c, &c->key, n)) || (rc = dalloc(c, &c->hist, c->update_words)) ||
        (rc = dalloc(c, &c->lookback, (size_t)kMaxPasses * c->sort_region)) ||
        (rc = dalloc(c, &c->sort_dirty, (size_t)kMaxPasses)) ||
        (rc = dalloc(c, &c->tickets, (size_t)kMaxPasses)) || (rc = dalloc(c, &c->a_key, n)) || (rc = dalloc(c, &c->a_val, n)) ||
        (rc = dalloc(c, &c->b_key[0], n)) || (rc = dalloc(c, &c->b_key[1], n)) || (rc = dalloc(c, &c->b_val[0], n)) ||
        (rc = dalloc(c, &c->b_val[1], n)) || (rc = dalloc(c, &c->ab_counts, 2)) ||
        (rc = dalloc(c, &c->merge_split, (size_t)merge_tiles(c->n) + 1)) || (rc = dalloc(c, &c->sorted_dev, 1)) ||
        (rc = dalloc(c, &c->nbr_count, n)) || (rc = dalloc(c, &c->pairs, kPairBins)) || (rc = dalloc(c, &c->err, 1)) ||
        (rc = dalloc(c, &c->check, 1)) || (rc = dalloc(c, &c->bounds_dev, 2)))
        return bail(rc);
    for (int b = 0; b < 2; b++) {
        if ((rc = dalloc(c, &c->kstart_b[b], c->num_keys + 1)) ||
            (rc = dalloc(c, &c->kstart_chunks_b[b], kstart_chunks(c->num_keys))) ||
            (rc = dalloc(c, &c->kstart_chunk_count_b[b], 1)) || (rc = dalloc(c, &c->sorted_pos_b[b], n)))
            return bail(rc);
    }
    c->mark_ticket = c->hist + (size_t)kMaxPasses * kRadix;
    c->mark_lookback = reinterpret_cast<unsigned long long*>(c->hist + (size_t)kMaxPasses * kRadix + 2u);
    use_index_buffers(c, 0);
    if (p.cap > 0) {
        size_t blocks = (n + kQueryThreads - 1) / kQueryThreads;
        if ((rc = dalloc(c, &c->nbr_list, blocks * kQueryThreads * (size_t)p.cap))) return bail(rc);
    }

    // ---- map upload (connections + one pad entry equal to the last) ----
    std::vector<uint32_t> conn(c->C + 1);
    if (c->C) std::memcpy(conn.data(), map->connections, sizeof(uint32_t) * c->C);
    conn[c->C] = c->C ? map->connections[c->C - 1] : 0u;
    e = cudaMemcpy(c->road_pos, map->road_pos, sizeof(float4) * c->R, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->road_conn, map->road_conn, sizeof(uint4) * c->R, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->conn, conn.data(), sizeof(uint32_t) * (c->C + 1), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->err, 0, sizeof(uint32_t), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->sorted_dev, 0, sizeof(unsigned long long), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->lookback, 0, sizeof(uint32_t) * kMaxPasses * c->sort_region, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->tickets, 0, sizeof(uint32_t) * kMaxPasses, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->sort_dirty, 0, sizeof(uint32_t) * kMaxPasses, c->stream);
    // the index buffers start zeroed (every slot and key in range), so even an index
    // update that was cut short leaves nothing out of range behind
    for (int b = 0; b < 2 && e == cudaSuccess; b++) {
        e = cudaMemsetAsync(c->sk[b], 0, sizeof(uint32_t) * std::max<size_t>(n, 1), c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->sv[b], 0, sizeof(uint32_t) * std::max<size_t>(n, 1), c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->kstart_b[b], 0, sizeof(uint32_t) * (c->num_keys + 1), c->stream);
    }
    for (int b = 0; b < 2 && e == cudaSuccess; b++) {
        e = cudaMemsetAsync(c->st[b].pos, 0, sizeof(float2) * std::max<size_t>(n, 1), c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->st[b].head, 0, sizeof(uint32_t) * std::max<size_t>(n, 1), c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->st[b].rng, 0, sizeof(uint4) * std::max<size_t>(n, 1), c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->st[b].speed, 0, sizeof(float) * std::max<size_t>(n, 1), c->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(c->st[b].slot_id, 0, sizeof(uint32_t) * std::max<size_t>(n, 1), c->stream);
    }
    if (e == cudaSuccess) e = configure_kernels(p.cap);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return bail(cuda_fail(e, "context set-up"));
    c->step_blocks = step_blocks_for(c->device, c->n);
    *out = c;
    return MSIM_OK;
}

int msim_destroy(msim_ctx* c) {
    if (!c) return MSIM_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    free_all(c);
    delete c;
    return MSIM_OK;
}

int msim_init_entities(msim_ctx* c, const msim_init* init) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (!init) return fail(MSIM_ERR_INVALID, "init is NULL");
    if (init->placement > 1) return fail(MSIM_ERR_INVALID, "unknown placement");
    if (!std::isfinite(init->speed_min) || !std::isfinite(init->speed_max) || init->speed_max < init->speed_min)
        return fail(MSIM_ERR_INVALID, "need finite speed_min <= speed_max");
    c->cur = 0;
    {
        Prof p(c, K_INIT);
        CK(launch_init_entities(c->stream, c->dmap(), c->st[0], c->n, c->params.rng_kind, init->seed, init->placement,
                                init->speed_min, init->speed_max),
           "k_init");
    }
    return build_index(c);
}

int msim_set_entities(msim_ctx* c, const float* pos, const uint32_t* heading, const uint32_t* rng,
                      const float* speed) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (c->n && (!pos || !heading || !rng)) return fail(MSIM_ERR_INVALID, "pos, heading and rng are required");
    const size_t n = c->n;
    if (n == 0) return MSIM_OK;
    // upload into the spare state buffer; it becomes current once the headings are checked
    const int b = 1 - c->cur;
    EntityState& s = c->st[b];
    CK(cudaMemcpyAsync(s.head, heading, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, c->stream), "upload heading");
    CK(launch_check_roads(c->stream, s.head, c->n, c->R, c->check), "k_check_roads");
    CK(cudaMemcpyAsync(s.pos, pos, sizeof(float2) * n, cudaMemcpyHostToDevice, c->stream), "upload pos");
    CK(cudaMemcpyAsync(s.rng, rng, sizeof(uint4) * n, cudaMemcpyHostToDevice, c->stream), "upload rng");
    if (speed) {
        CK(cudaMemcpyAsync(s.speed, speed, sizeof(float) * n, cudaMemcpyHostToDevice, c->stream), "upload speed");
    } else {
        CK(launch_fill(c->stream, s.speed, c->n, 1.4f), "k_fill");  // SPEED, random_move.comp:750
    }
    uint32_t first_bad = 0;
    CK(cudaMemcpyAsync(&first_bad, c->check, sizeof(first_bad), cudaMemcpyDeviceToHost, c->stream), "read check");
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    if (first_bad != 0xffffffffu)
        return fail(MSIM_ERR_OOB, "heading of entity " + std::to_string(first_bad) + " names road " +
                                      std::to_string(heading[first_bad] & MSIM_HEADING_ROAD_MASK) + " of " +
                                      std::to_string(c->R));
    c->cur = b;
    // entity i starts in slot i.  No index is built here: the next neighbour tick
    // sorts from scratch, and re-orders the state into spatial order the tick after
    // (a re-ordering from the caller's arbitrary order is a random gather, as costly
    // as the upload itself; a caller that sets the state before every tick never
    // pays it).
    CK(launch_iota(c->stream, s.slot_id, c->n), "k_iota");
    reset_index(c);
    c->bounds_valid = false;
    c->slots_identity = true;
    return MSIM_OK;
}

int msim_set_road_factors(msim_ctx* c, const float* factors) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (!factors) return fail(MSIM_ERR_INVALID, "factors is NULL");
    double fmax = 0.0;
    for (uint32_t r = 0; r < c->R; r++) {
        if (!std::isfinite(factors[r])) return fail(MSIM_ERR_INVALID, "non-finite road factor");
        fmax = std::max(fmax, std::fabs((double)factors[r]));
    }
    if (!c->factor && (rc = dalloc(c, &c->factor, c->R))) return rc;
    CK(cudaMemcpyAsync(c->factor, factors, sizeof(float) * c->R, cudaMemcpyHostToDevice, c->stream), "upload factors");
    CK(cudaStreamSynchronize(c->stream), "sync");
    // ticks from here on move by the new factors: an index built before is not reused
    c->max_factor = fmax;
    c->bounds_valid = false;
    if (c->reuse_ticks > 0) c->reuse_ticks = -1;
    return MSIM_OK;
}

int msim_step(msim_ctx* c, uint32_t ticks, uint32_t flags) {
    NvtxRange range("msim_step");
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (flags & ~MSIM_STEP_NEIGHBOURS) return fail(MSIM_ERR_INVALID, "unknown step flags");
    if (c->n == 0) {
        c->tick += ticks;
        return MSIM_OK;
    }
    c->state_free_event = false;
    if (flags & MSIM_STEP_NEIGHBOURS) {
        for (uint32_t t = 0; t < ticks; t++) {
            rc = neighbour_tick(c);
            if (rc != MSIM_OK) {
                // a launch of the tick failed: the index is rebuilt from scratch by the
                // next neighbour tick; the move of this tick may or may not have run
                join_query(c);
                c->chain_broken = true;
                reset_index(c);
                return rc;
            }
            c->tick++;
        }
        return join_query(c);  // later work on the context's stream sees the last query
    }
    // move only: up to 256 ticks per launch with the state in registers
    uint32_t left = ticks;
    while (left) {
        uint32_t t = std::min<uint32_t>(left, 256u);
        Prof p(c, K_STEP_MULTI);
        CKL(p, launch_step(c->stream, step_args(c, t, false)), "k_step_multi");
        left -= t;
        c->tick += t;
        if (c->reuse_ticks >= 0) c->reuse_ticks += t;  // moved without an index update
    }
    return MSIM_OK;
}

int msim_sync(msim_ctx* c) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    return sync_and_check(c);
}

int msim_get_state(msim_ctx* c, float* pos, uint32_t* heading, uint32_t* rng, float* speed) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    const size_t n = c->n;
    if (n == 0) return sync_and_check(c);
    if ((rc = ensure_stage(c, n * (sizeof(float2) + sizeof(uint32_t) + sizeof(uint4) + sizeof(float)))) != MSIM_OK)
        return rc;
    char* b = static_cast<char*>(c->stage);
    uint4* d_rng = reinterpret_cast<uint4*>(b);
    float2* d_pos = reinterpret_cast<float2*>(b + n * sizeof(uint4));
    uint32_t* d_head = reinterpret_cast<uint32_t*>(b + n * (sizeof(uint4) + sizeof(float2)));
    float* d_speed = reinterpret_cast<float*>(b + n * (sizeof(uint4) + sizeof(float2) + sizeof(uint32_t)));
    {
        Prof p(c, K_EXPORT);
        CK(launch_export_state(c->stream, cur_state(c), c->n, pos ? d_pos : nullptr, heading ? d_head : nullptr,
                               rng ? d_rng : nullptr, speed ? d_speed : nullptr),
           "k_export_state");
    }
    if (pos) CK(cudaMemcpyAsync(pos, d_pos, sizeof(float2) * n, cudaMemcpyDeviceToHost, c->stream), "download pos");
    if (heading)
        CK(cudaMemcpyAsync(heading, d_head, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, c->stream), "download heading");
    if (rng) CK(cudaMemcpyAsync(rng, d_rng, sizeof(uint4) * n, cudaMemcpyDeviceToHost, c->stream), "download rng");
    if (speed) CK(cudaMemcpyAsync(speed, d_speed, sizeof(float) * n, cudaMemcpyDeviceToHost, c->stream), "download speed");
    return sync_and_check(c);
}

int msim_get_neighbours(msim_ctx* c, uint32_t* count, uint32_t* idx) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (!count) return fail(MSIM_ERR_INVALID, "count is NULL");
    if (!c->have_nbr) return fail(MSIM_ERR_INVALID, "no neighbour tick has run since the entities were set");
    const size_t n = c->n, cap = c->params.cap;
    if (n == 0) return MSIM_OK;
    const bool want_idx = idx && cap;
    if ((rc = ensure_stage(c, n * sizeof(uint32_t) * (1 + (want_idx ? cap : 0)))) != MSIM_OK) return rc;
    uint32_t* d_count = static_cast<uint32_t*>(c->stage);
    uint32_t* d_idx = want_idx ? d_count + n : nullptr;
    {
        Prof p(c, K_EXPORT);
        CK(launch_export_neighbours(c->stream, c->query_slot, cur_state(c).slot_id, c->nbr_count, c->nbr_list,
                                    c->n, c->params.cap, d_count, d_idx),
           "k_export_nbr");
    }
    CK(cudaMemcpyAsync(count, d_count, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, c->stream), "download counts");
    if (want_idx)
        CK(cudaMemcpyAsync(idx, d_idx, sizeof(uint32_t) * n * cap, cudaMemcpyDeviceToHost, c->stream),
           "download neighbours");
    return sync_and_check(c);
}

int msim_tick_host(msim_ctx* c, const float* in_pos, const uint32_t* in_heading, const uint32_t* in_rng,
                   const float* in_speed, uint32_t flags, float* out_pos, uint32_t* out_heading, uint32_t* out_rng,
                   uint32_t* out_count, uint32_t* out_idx) {
    NvtxRange range("msim_tick_host");
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (flags & ~MSIM_STEP_NEIGHBOURS) return fail(MSIM_ERR_INVALID, "unknown step flags");
    const bool nbr = (flags & MSIM_STEP_NEIGHBOURS) != 0;
    if ((out_count || out_idx) && !nbr) return fail(MSIM_ERR_INVALID, "neighbour outputs need MSIM_STEP_NEIGHBOURS");
    const uint32_t n = c->n;
    if (n && (!in_pos || !in_heading || !in_rng)) return fail(MSIM_ERR_INVALID, "pos, heading and rng are required");
    if (n == 0) {
        c->tick++;
        return MSIM_OK;
    }
    if (!c->up) {
        CK(cudaStreamCreateWithFlags(&c->up, cudaStreamNonBlocking), "cudaStreamCreate");
        CK(cudaStreamCreateWithFlags(&c->down, cudaStreamNonBlocking), "cudaStreamCreate");
        CK(cudaEventCreateWithFlags(&c->ev_start, cudaEventDisableTiming), "cudaEventCreate");
        CK(cudaEventCreateWithFlags(&c->ev_disp, cudaEventDisableTiming), "cudaEventCreate");
        CK(cudaEventCreateWithFlags(&c->ev_query, cudaEventDisableTiming), "cudaEventCreate");
        CK(cudaEventCreateWithFlags(&c->ev_state_free, cudaEventDisableTiming), "cudaEventCreate");
        for (uint32_t k = 0; k < kHostChunks; k++) {
            CK(cudaEventCreateWithFlags(&c->ev_up[k], cudaEventDisableTiming), "cudaEventCreate");
            CK(cudaEventCreateWithFlags(&c->ev_moved[k], cudaEventDisableTiming), "cudaEventCreate");
        }
    }
    // The spare state buffer receives the upload; earlier work (a re-ordering that
    // read it, a query still running) finishes first.
    if ((rc = join_query(c)) != MSIM_OK) return rc;
    const int old = c->cur;
    const int b = 1 - old;
    EntityState& s = c->st[b];
    // The previous index stays a valid starting order for an incremental update when
    // its slots already held entity ids (the previous call was a host tick, or a set
    // followed by one tick): the new state goes to the same slots.
    const bool old_slots_identity = c->slots_identity;
    const bool use_inc = nbr && c->incremental && c->sorted_key && c->slots_identity;
    // Skin query: when the current index was built from the keys of the state this
    // tick starts from (the previous call was a neighbour host tick and nothing moved
    // or set the state since), this tick's query reads that index with every box
    // widened by the tick's largest displacement d (an entity within the radius of
    // another now lay within radius + d of it when the index was built, in each
    // coordinate).  The move measures d; the new positions are gathered into the
    // index's order chunk by chunk behind the uploads; the index update for the new
    // state then runs after the query, beside the downloads and the next call's
    // uploads.  A d above kWidenLimit of the reach (host edits between ticks, large
    // steps) takes the usual order: index update, then query.
    const bool state_free_event = c->state_free_event;
    bool skin = c->reuse && use_inc && c->reuse_ticks == 0 && c->grid.reach > 0.f && ensure_skin(c);
    c->reuse_ticks = -1;
    c->bounds_valid = false;  // speeds and positions come from the host
    c->state_free_event = false;
    // In place (the same page-locked arrays for heading and RNG in and out): they
    // already hold every value the tick leaves unchanged, so the move kernel writes the
    // headings and RNG states that change (entities at a road end, a few per thousand
    // per tick) straight into them through their device mapping, and only positions
    // are downloaded.
    uint32_t* dev_head = nullptr;
    uint4* dev_rng = nullptr;
    if (out_heading && static_cast<const void*>(out_heading) == static_cast<const void*>(in_heading) && out_rng &&
        static_cast<const void*>(out_rng) == static_cast<const void*>(in_rng)) {
        dev_head = static_cast<uint32_t*>(mapped_host(out_heading));
        dev_rng = static_cast<uint4*>(mapped_host(out_rng));
        if (!dev_head || !dev_rng || (reinterpret_cast<uintptr_t>(dev_rng) & 15u)) {
            dev_head = nullptr;
            dev_rng = nullptr;
        }
    }
    const bool in_place = dev_head != nullptr;
    CK(cudaMemsetAsync(c->check, 0xff, sizeof(uint32_t), c->stream), "memset check");
    if (nbr && !use_inc) CK(cudaMemsetAsync(c->hist, 0, sizeof(uint32_t) * kMaxPasses * kRadix, c->stream), "memset hist");
    if (use_inc && (rc = clear_update_scratch(c)) != MSIM_OK) return rc;
    if (skin) CK(cudaMemsetAsync(c->disp, 0, sizeof(uint32_t), c->stream), "memset displacement");
    // entity i in slot i (for later calls; this tick's query and export take the slot
    // as the id): written first, beside the first chunk's upload
    CK(launch_iota(c->stream, s.slot_id, n), "k_iota");
    if (state_free_event) {
        // the last read of the spare buffer was recorded before the previous call's
        // index update, which so runs beside these uploads
        CK(cudaStreamWaitEvent(c->up, c->ev_state_free, 0), "cudaStreamWaitEvent");
    } else {
        CK(cudaEventRecord(c->ev_start, c->stream), "cudaEventRecord");
        CK(cudaStreamWaitEvent(c->up, c->ev_start, 0), "cudaStreamWaitEvent");
    }

    // chunk k: upload (up) -> check headings, move, key, digit counts (stream) ->
    // download of the moved state (down); chunk k's download overlaps chunk k+1's upload
    const uint32_t chunk = std::max<uint32_t>(kHostChunkMin, (n + kHostChunks - 1) / kHostChunks);
    uint32_t k = 0;
    uint32_t last_lo = 0, last_cnt = 0;
    for (uint32_t lo = 0; lo < n; lo += chunk, k++) {
        const uint32_t cnt = std::min(chunk, n - lo);
        CK(cudaMemcpyAsync(s.head + lo, in_heading + lo, sizeof(uint32_t) * cnt, cudaMemcpyHostToDevice, c->up),
           "upload heading");
        CK(cudaMemcpyAsync(s.pos + lo, in_pos + 2 * (size_t)lo, sizeof(float2) * cnt, cudaMemcpyHostToDevice, c->up),
           "upload pos");
        CK(cudaMemcpyAsync(s.rng + lo, in_rng + 4 * (size_t)lo, sizeof(uint4) * cnt, cudaMemcpyHostToDevice, c->up),
           "upload rng");
        if (in_speed)
            CK(cudaMemcpyAsync(s.speed + lo, in_speed + lo, sizeof(float) * cnt, cudaMemcpyHostToDevice, c->up),
               "upload speed");
        CK(cudaEventRecord(c->ev_up[k], c->up), "cudaEventRecord");
        CK(cudaStreamWaitEvent(c->stream, c->ev_up[k], 0), "cudaStreamWaitEvent");
        if (!in_speed) CK(launch_fill(c->stream, s.speed + lo, cnt, 1.4f), "k_fill");  // SPEED, random_move.comp:750
        if (!skin)  // (the skin path's move checks the headings itself)
            CK(launch_check_roads_range(c->stream, s.head, lo, cnt, c->R, c->check), "k_check_roads");
        {
            Prof p(c, K_STEP);
            StepLaunch a = step_args(c, 1, nbr);
            a.st.pos = s.pos + lo;
            a.st.head = s.head + lo;
            a.st.rng = s.rng + lo;
            a.st.speed = s.speed + lo;
            a.st.slot_id = s.slot_id + lo;
            a.n = cnt;
            a.key = nbr ? c->key + lo : nullptr;
            if (use_inc) a.hist = nullptr;  // the changed keys' digits are counted by k_mark
            a.blocks = std::min<int>(c->step_blocks, (int)((cnt + kStepThreads - 1) / kStepThreads));
            a.host_head = dev_head;
            a.host_rng = dev_rng;
            a.id_base = lo;
            if (skin) {  // displacement against the positions the current index was built from
                a.index_pos = c->st[old].pos + lo;
                a.disp_max = c->disp;
                a.first_bad = c->check;
            }
            CK(launch_step(c->stream, a), "k_step");
        }
        CK(cudaEventRecord(c->ev_moved[k], c->stream), "cudaEventRecord");
        CK(cudaStreamWaitEvent(c->down, c->ev_moved[k], 0), "cudaStreamWaitEvent");
        if (out_pos)
            CK(cudaMemcpyAsync(out_pos + 2 * (size_t)lo, s.pos + lo, sizeof(float2) * cnt, cudaMemcpyDeviceToHost,
                               c->down),
               "download pos");
        if (!in_place) {  // headings and RNG states in place: written by the move kernel
            if (out_heading)
                CK(cudaMemcpyAsync(out_heading + lo, s.head + lo, sizeof(uint32_t) * cnt, cudaMemcpyDeviceToHost,
                                   c->down),
                   "download heading");
            if (out_rng)
                CK(cudaMemcpyAsync(out_rng + 4 * (size_t)lo, s.rng + lo, sizeof(uint4) * cnt,
                                   cudaMemcpyDeviceToHost, c->down),
                   "download rng");
        }
        last_lo = lo;
        last_cnt = cnt;
        if (skin && lo + cnt < n) {  // the last chunk's gather runs while the host reads d
            Prof p(c, K_GATHER);
            CK(launch_gather_chunk(c->stream, c->sorted_slot, n, lo, cnt, s.pos, c->skin_pos), "k_gather_chunk");
        }
    }
    c->cur = b;
    c->slots_identity = true;
    TileGrid skin_grid = c->grid;
    if (skin) {
        CK(cudaMemcpyAsync(c->disp_host, c->disp, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream),
           "read displacement");
        CK(cudaEventRecord(c->ev_disp, c->stream), "cudaEventRecord");
        {
            Prof p(c, K_GATHER);
            CK(launch_gather_chunk(c->stream, c->sorted_slot, n, last_lo, last_cnt, s.pos, c->skin_pos),
               "k_gather_chunk");
        }
        CK(cudaEventSynchronize(c->ev_disp), "cudaEventSynchronize");
        float d = 0.f;
        std::memcpy(&d, c->disp_host, sizeof(d));
        c->last_disp = d;
        skin = d <= kWidenLimit * c->grid.reach;  // false for +inf (a non-finite position)
        if (skin) {
            // widened reach, rounded up: the displacement was measured with one rounding
            const double r = (double)c->grid.reach + (double)d * (1.0 + 0x1p-20);
            float rf = (float)r;
            if ((double)rf < r) rf = std::nextafter(rf, INFINITY);
            skin_grid.reach = rf;
        }
    }
    const bool want_idx = nbr && out_idx && c->params.cap;
    const size_t cap = c->params.cap;
    uint32_t* d_count = nullptr;
    if (nbr && (out_count || out_idx)) {
        if ((rc = ensure_stage(c, (size_t)n * sizeof(uint32_t) * (1 + (want_idx ? cap : 0)))) != MSIM_OK) return rc;
        d_count = static_cast<uint32_t*>(c->stage);
    }
    uint32_t* d_idx = want_idx ? d_count + n : nullptr;
    // the neighbour downloads go on `dl`: the context's stream, or (skin query) the
    // download stream, so the index update can follow the query on the context's stream
    cudaStream_t dl = c->stream;
    if (nbr && skin) {
        // slots hold entity ids: the query writes the counts by id itself
        if ((rc = run_query(c, false, d_count, c->skin_pos, &skin_grid)) != MSIM_OK) return rc;
        if (want_idx) {
            Prof p(c, K_EXPORT);
            CK(launch_export_neighbours(c->stream, c->query_slot, nullptr, c->nbr_count, c->nbr_list, n,
                                        c->params.cap, d_count, d_idx),
               "k_export_nbr");
        }
        // the status as the query left it, before the index update below can raise one
        CK(cudaMemcpyAsync(c->disp_host + 1, c->err, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream),
           "read device status");
        CK(cudaEventRecord(c->ev_query, c->stream), "cudaEventRecord");
        CK(cudaStreamWaitEvent(c->down, c->ev_query, 0), "cudaStreamWaitEvent");
        // nothing after this point reads the spare state buffer: the next call's uploads
        // may start while the index update below runs
        CK(cudaEventRecord(c->ev_state_free, c->stream), "cudaEventRecord");
        dl = c->down;
    } else if (nbr) {
        if (use_inc) {
            if ((rc = incremental_update(c, true, false)) != MSIM_OK) return rc;
        } else {
            reset_index(c);
            if ((rc = sort_keys(c)) != MSIM_OK || (rc = key_start_table(c)) != MSIM_OK) return rc;
        }
        // slots hold entity ids here: the query writes the counts by id itself, so with
        // counts alone no export pass runs between the query and their download
        if ((rc = run_query(c, false, d_count)) != MSIM_OK) return rc;
        if (want_idx) {
            Prof p(c, K_EXPORT);
            CK(launch_export_neighbours(c->stream, c->query_slot, nullptr, c->nbr_count, c->nbr_list, n,
                                        c->params.cap, d_count, d_idx),
               "k_export_nbr");
        }
    } else {
        reset_index(c);
    }
    if (out_count) CK(cudaMemcpyAsync(out_count, d_count, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, dl), "download counts");
    if (want_idx)
        CK(cudaMemcpyAsync(out_idx, d_idx, sizeof(uint32_t) * n * cap, cudaMemcpyDeviceToHost, dl),
           "download neighbours");
    // the index of the new state for the next call (no sorted positions: its query
    // gathers its own); with the skin query this runs after the query, off the host's path
    if (nbr && skin && (rc = incremental_update(c, false, false)) != MSIM_OK) return rc;
    c->tick++;
    uint32_t first_bad = 0;
    // read after the query: the heading checks of every chunk ran before it
    CK(cudaMemcpyAsync(&first_bad, c->check, sizeof(first_bad), cudaMemcpyDeviceToHost, dl), "read check");
    CK(cudaStreamSynchronize(c->down), "cudaStreamSynchronize");
    if (!skin) CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    const uint32_t status = skin ? c->disp_host[1] : 0u;
    if (first_bad != 0xffffffffu) {  // as msim_set_entities: the previous state stays
        CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
        c->cur = old;
        reset_index(c);
        c->slots_identity = old_slots_identity;
        c->tick--;
        CK(cudaMemsetAsync(c->err, 0, sizeof(uint32_t), c->stream), "clear device status");
        CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
        return fail(MSIM_ERR_OOB, "heading of entity " + std::to_string(first_bad) + " names road " +
                                      std::to_string(in_heading[first_bad] & MSIM_HEADING_ROAD_MASK) + " of " +
                                      std::to_string(c->R));
    }
    if (skin) {
        // a status raised before the query (e.g. by the previous call's index update):
        // reported now, after everything on the context's stream
        if (status) return sync_and_check(c);
        c->reuse_ticks = 0;
        c->state_free_event = true;
        c->host_ticks++;
        c->skin_queries++;
        return MSIM_OK;
    }
    rc = sync_and_check(c);
    if (rc == MSIM_OK) {
        c->reuse_ticks = nbr ? 0 : -1;  // the index was built from this state
        c->host_ticks++;
    }
    return rc;
}

int msim_get_collision_pairs(msim_ctx* c, uint64_t* pairs) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (!pairs) return fail(MSIM_ERR_INVALID, "pairs is NULL");
    if (!c->have_nbr) return fail(MSIM_ERR_INVALID, "no neighbour tick has run since the entities were set");
    unsigned long long h[kPairBins];
    CK(cudaMemcpyAsync(h, c->pairs, sizeof(h), cudaMemcpyDeviceToHost, c->stream), "download pairs");
    rc = sync_and_check(c);
    uint64_t sum = 0;
    for (uint32_t b = 0; b < kPairBins; b++) sum += h[b];
    *pairs = sum / 2u;  // the bins hold the sum of all counts: every pair from both ends
    return rc;
}

int msim_export_entities_aos(msim_ctx* c, void* out, size_t n) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (!out && n) return fail(MSIM_ERR_INVALID, "out is NULL");
    if (n != c->n) return fail(MSIM_ERR_INVALID, "n must equal num_entities");
    if (n == 0) return MSIM_OK;
    if ((rc = ensure_stage(c, n * 64)) != MSIM_OK) return rc;
    {
        Prof p(c, K_EXPORT);
        CK(launch_export_aos(c->stream, c->dmap(), cur_state(c), c->n, c->params.dt,
                             c->have_nbr ? c->query_slot : nullptr, c->have_nbr ? c->nbr_count : nullptr, c->stage),
           "k_export_aos");
    }
    CK(cudaMemcpyAsync(out, c->stage, n * 64, cudaMemcpyDeviceToHost, c->stream), "download entities");
    return sync_and_check(c);
}

int msim_export_quad_tree(msim_ctx* c, uint32_t max_depth, uint32_t node_cap, void* nodes, uint32_t node_capacity,
                          void* links, uint32_t* nodes_used) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    std::vector<float> pos((size_t)c->n * 2);
    rc = msim_get_state(c, pos.data(), nullptr, nullptr, nullptr);
    if (rc != MSIM_OK) return rc;
    return build_quad_tree(pos.data(), c->n, c->world_w, c->world_h, max_depth, node_cap, nodes, node_capacity, links,
                           nodes_used);
}

int msim_get_tick(msim_ctx* c, uint64_t* tick) {
    if (!c || !tick) return fail(MSIM_ERR_INVALID, "NULL argument");
    *tick = c->tick;
    return MSIM_OK;
}

// Snapshot file: "MSIMSNP1", then u32 num_entities, num_roads, num_connections,
// rng_kind, u64 tick, then by entity id pos (2 f32), heading (u32), rng (4 u32) and
// speed (f32) arrays, little-endian as the host writes them.
namespace {
constexpr char kSnapMagic[8] = {'M', 'S', 'I', 'M', 'S', 'N', 'P', '1'};
struct SnapHeader {
    char magic[8];
    uint32_t n, roads, conns, rng_kind;
    uint64_t tick;
};
}  // namespace

int msim_save_state(msim_ctx* c, const char* path) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (!path) return fail(MSIM_ERR_INVALID, "path is NULL");
    const size_t n = c->n;
    std::vector<float> pos(2 * n), speed(n);
    std::vector<uint32_t> head(n), rng(4 * n);
    if ((rc = msim_get_state(c, pos.data(), head.data(), rng.data(), speed.data())) != MSIM_OK) return rc;
    SnapHeader h{};
    std::memcpy(h.magic, kSnapMagic, sizeof(h.magic));
    h.n = c->n;
    h.roads = c->R;
    h.conns = c->C;
    h.rng_kind = c->params.rng_kind;
    h.tick = c->tick;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(MSIM_ERR_IO, std::string("cannot write ") + path);
    bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 && std::fwrite(pos.data(), sizeof(float), 2 * n, f) == 2 * n &&
              std::fwrite(head.data(), sizeof(uint32_t), n, f) == n &&
              std::fwrite(rng.data(), sizeof(uint32_t), 4 * n, f) == 4 * n &&
              std::fwrite(speed.data(), sizeof(float), n, f) == n;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? MSIM_OK : fail(MSIM_ERR_IO, std::string("short write to ") + path);
}

int msim_load_state(msim_ctx* c, const char* path) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (!path) return fail(MSIM_ERR_INVALID, "path is NULL");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(MSIM_ERR_IO, std::string("cannot read ") + path);
    SnapHeader h{};
    if (std::fread(&h, sizeof(h), 1, f) != 1 || std::memcmp(h.magic, kSnapMagic, sizeof(h.magic)) != 0) {
        std::fclose(f);
        return fail(MSIM_ERR_INVALID, std::string(path) + " is not a snapshot");
    }
    if (h.n != c->n || h.roads != c->R || h.conns != c->C || h.rng_kind != c->params.rng_kind) {
        std::fclose(f);
        return fail(MSIM_ERR_INVALID, "snapshot of another configuration (entities, map or RNG differ)");
    }
    const size_t n = c->n;
    std::vector<float> pos(2 * n), speed(n);
    std::vector<uint32_t> head(n), rng(4 * n);
    const bool ok = std::fread(pos.data(), sizeof(float), 2 * n, f) == 2 * n &&
                    std::fread(head.data(), sizeof(uint32_t), n, f) == n &&
                    std::fread(rng.data(), sizeof(uint32_t), 4 * n, f) == 4 * n &&
                    std::fread(speed.data(), sizeof(float), n, f) == n;
    std::fclose(f);
    if (!ok) return fail(MSIM_ERR_IO, std::string("truncated snapshot ") + path);
    if ((rc = msim_set_entities(c, pos.data(), head.data(), rng.data(), speed.data())) != MSIM_OK) return rc;
    c->tick = h.tick;
    return MSIM_OK;
}

int msim_get_launch_count(msim_ctx* c, uint64_t* launches) {
    if (!c || !launches) return fail(MSIM_ERR_INVALID, "NULL argument");
    *launches = c->launch_count;
    return MSIM_OK;
}

int msim_set_tick_timing(msim_ctx* c, int enable) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (enable) {
        for (int k = 0; k < 3; k++)
            if (!c->ev_tick[k]) CK(cudaEventCreate(&c->ev_tick[k]), "cudaEventCreate");
    }
    c->tick_timing = enable != 0;
    c->tick_recorded = false;
    return MSIM_OK;
}

int msim_get_tick_times(msim_ctx* c, float* update_ms, float* collision_ms) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (!c->tick_recorded) return fail(MSIM_ERR_INVALID, "no neighbour tick timed since tick timing was enabled");
    CK(cudaEventSynchronize(c->ev_tick[2]), "cudaEventSynchronize");
    float u = 0.f, q = 0.f;
    CK(cudaEventElapsedTime(&u, c->ev_tick[0], c->ev_tick[1]), "cudaEventElapsedTime");
    CK(cudaEventElapsedTime(&q, c->ev_tick[1], c->ev_tick[2]), "cudaEventElapsedTime");
    if (update_ms) *update_ms = u;
    if (collision_ms) *collision_ms = q;
    return MSIM_OK;
}

int msim_set_device(int device) {
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceCount");
    if (device < 0 || device >= count)
        return fail(MSIM_ERR_INVALID, "device " + std::to_string(device) + " of " + std::to_string(count));
    CK(cudaSetDevice(device), "cudaSetDevice");
    return MSIM_OK;
}

int msim_set_wait_limit(msim_ctx* c, uint32_t polls) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    c->spin_limit = polls ? polls : kDefaultSpinLimit;
    return MSIM_OK;
}

int msim_debug_inject(msim_ctx* c, uint32_t fault, uint32_t arg) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (fault > MSIM_FAULT_LAUNCH) return fail(MSIM_ERR_INVALID, "unknown fault");
    c->fault = fault;
    c->fault_arg = arg;
    return MSIM_OK;
}

int msim_debug_fail_device_alloc(int64_t after) {
    g_alloc_budget.store(after < 0 ? -1 : (long long)after);
    return MSIM_OK;
}

int msim_set_profiling(msim_ctx* c, int enable) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    c->profiling = enable != 0;
    return MSIM_OK;
}

int msim_reset_kernel_stats(msim_ctx* c) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    rc = drain_profile(c);
    for (uint32_t k = 0; k < K_COUNT; k++) {
        c->launches[k] = 0;
        c->ms[k] = 0.0;
    }
    c->sorted_host = 0;
    c->index_updates = 0;
    c->host_ticks = 0;
    c->skin_queries = 0;
    CK(cudaMemsetAsync(c->sorted_dev, 0, sizeof(unsigned long long), c->stream), "memset sort stats");
    return rc;
}

int msim_get_host_tick_stats(msim_ctx* c, uint64_t* host_ticks, uint64_t* skin_queries, float* last_displacement) {
    if (!c) return fail(MSIM_ERR_INVALID, "context is NULL");
    if (host_ticks) *host_ticks = c->host_ticks;
    if (skin_queries) *skin_queries = c->skin_queries;
    if (last_displacement) *last_displacement = c->last_disp;
    return MSIM_OK;
}

int msim_get_sort_stats(msim_ctx* c, uint64_t* index_updates, uint64_t* sorted_entries) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    unsigned long long dev = 0;
    CK(cudaMemcpyAsync(&dev, c->sorted_dev, sizeof(dev), cudaMemcpyDeviceToHost, c->stream), "read sort stats");
    CK(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    if (index_updates) *index_updates = c->index_updates;
    if (sorted_entries) *sorted_entries = c->sorted_host + dev;
    return MSIM_OK;
}

int msim_get_kernel_stats(msim_ctx* c, uint32_t kernel, uint64_t* launches, double* total_ms) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (kernel >= K_COUNT) return fail(MSIM_ERR_INVALID, "unknown kernel id");
    rc = drain_profile(c);
    if (rc != MSIM_OK) return rc;
    if (launches) *launches = c->launches[kernel];
    if (total_ms) *total_ms = c->ms[kernel];
    return MSIM_OK;
}

int msim_timer_begin(msim_ctx* c) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    CK(cudaEventRecord(c->t0, c->stream), "cudaEventRecord");
    c->timer_open = true;
    return MSIM_OK;
}

int msim_timer_end(msim_ctx* c, float* ms) {
    int rc = check_ctx(c);
    if (rc != MSIM_OK) return rc;
    if (!c->timer_open || !ms) return fail(MSIM_ERR_INVALID, "timer not started or ms is NULL");
    CK(cudaEventRecord(c->t1, c->stream), "cudaEventRecord");
    CK(cudaEventSynchronize(c->t1), "cudaEventSynchronize");
    CK(cudaEventElapsedTime(ms, c->t0, c->t1), "cudaEventElapsedTime");
    c->timer_open = false;
    return MSIM_OK;
}

int msim_host_alloc(size_t bytes, void** out) {
    if (!out) return fail(MSIM_ERR_INVALID, "out is NULL");
    *out = nullptr;
    cudaError_t e = cudaMallocHost(out, bytes ? bytes : 1);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(MSIM_ERR_NOMEM, std::string("cudaMallocHost failed: ") + cudaGetErrorString(e));
    }
    return MSIM_OK;
}

int msim_host_free(void* ptr) {
    if (!ptr) return MSIM_OK;
    cudaError_t e = cudaFreeHost(ptr);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFreeHost");
    return MSIM_OK;
}

int msim_get_info(msim_ctx* c, msim_info* out) {
    if (!c || !out) return fail(MSIM_ERR_INVALID, "NULL argument");
    out->num_entities = c->n;
    out->num_roads = c->R;
    out->num_connections = c->C;
    out->tiles_x = c->grid.tiles_x;
    out->tiles_y = c->grid.tiles_y;
    out->key_bits = 2 * c->grid.bits + c->grid.ybits;
    out->sort_passes = c->passes;
    out->resort_interval = c->resort;
    out->cell_size = 1.f / c->grid.inv_cell;
    out->cap = c->params.cap;
    out->device_bytes = c->device_bytes;
    return MSIM_OK;
}

}  // extern "C"
