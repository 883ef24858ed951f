// Batched ensemble: many independent movement-sim instances (each its own road
// graph and entities) advanced together by one persistent kernel launch.
//
// All instances' entity state is concatenated (structure of arrays) and so are
// their road tables (road_pos, road_conn, connections + one pad entry each).  The
// host cuts every instance into tiles of entities; each tile is a work item with
// an entities-per-thread factor.  A persistent grid (a few blocks per SM) pulls
// items through an atomic ticket and runs all requested ticks of a tile with the
// state in registers.  The per-entity math is step_entity, the same function as
// the single-instance path, so every instance's result is bit-identical to
// running it alone.  The ticket reset and the launch are captured once per tick
// count into a CUDA graph and replayed.
//
// Schedules (block size; per size class the entities per thread and the tile
// size) come from msim_batch_tune, which times candidates on the instances
// themselves and can cache the choice in a JSON file.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <new>
#include <sstream>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "msim_internal.h"
#include "msim_kernels.cuh"

namespace msim {
namespace {

struct InstanceDesc {
    uint32_t road_base;
    uint32_t conn_base;
    uint32_t num_roads;
    uint32_t num_conn;
};

struct WorkItem {
    uint32_t instance;
    uint32_t begin;  // first entity (global index into the concatenated state)
    uint32_t count;
    uint32_t ept;    // entities per thread: 1, 2 or 4
};

struct BatchArgs {
    const float4* road_pos;
    const uint4* road_conn;
    const uint32_t* conn;
    const InstanceDesc* inst;
    const WorkItem* items;
    uint32_t num_items;
    uint32_t* ticket;
    float2* pos;
    uint32_t* head;
    uint4* rng;
    const float* speed;
    float dt;
    uint32_t ticks;
    uint32_t* err;
};

// E independent entities per thread, interleaved tick by tick so their
// dependency chains overlap.
template <int RNG, int E>
__device__ __forceinline__ void run_tile(const BatchArgs& a, const DeviceMap& m, const WorkItem& it) {
    const uint32_t span = blockDim.x * E;
    for (uint32_t off = 0; off < it.count; off += span) {
        float2 p[E];
        uint32_t h[E], h0[E];
        float sp[E];
        uint4 r[E];
        bool rl[E], rd[E], ok[E];
#pragma unroll
        for (int k = 0; k < E; k++) {
            const uint32_t local = off + threadIdx.x + k * blockDim.x;
            ok[k] = local < it.count;
            const uint32_t e = it.begin + (ok[k] ? local : 0u);
            p[k] = a.pos[e];
            h[k] = h0[k] = a.head[e];
            sp[k] = a.speed[e];
            r[k] = make_uint4(0u, 0u, 0u, 0u);
            rl[k] = rd[k] = false;
        }
        for (uint32_t t = 0; t < a.ticks; t++) {
#pragma unroll
            for (int k = 0; k < E; k++) {
                const uint32_t e = it.begin + off + threadIdx.x + k * blockDim.x;
                if (ok[k]) step_entity<RNG>(m, a.dt, sp[k], p[k], h[k], r[k], rl[k], rd[k], a.rng + e, a.err);
            }
        }
#pragma unroll
        for (int k = 0; k < E; k++) {
            if (!ok[k]) continue;
            const uint32_t e = it.begin + off + threadIdx.x + k * blockDim.x;
            a.pos[e] = p[k];
            if (h[k] != h0[k]) a.head[e] = h[k];
            if (rd[k]) a.rng[e] = r[k];
        }
    }
}

// EMAX: the largest entities-per-thread count of the schedule.  Each value is its own
// kernel, so a schedule of one entity per thread does not pay the registers of the
// four-entity path (72 registers and 43 % of the warps resident with all three paths
// in one kernel).
template <int RNG, int EMAX>
__global__ void k_batch_step(BatchArgs a) {
    __shared__ uint32_t s_item;
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(a.ticket, 1u);
        __syncthreads();
        const uint32_t i = s_item;
        if (i >= a.num_items) return;
        const WorkItem it = a.items[i];
        const InstanceDesc d = a.inst[it.instance];
        DeviceMap m;
        m.road_pos = a.road_pos + d.road_base;
        m.road_conn = a.road_conn + d.road_base;
        m.conn = a.conn + d.conn_base;
        m.factor = nullptr;
        m.num_roads = d.num_roads;
        m.num_conn = d.num_conn;
        if (EMAX >= 4 && it.ept == 4) run_tile<RNG, 4>(a, m, it);
        else if (EMAX >= 2 && it.ept == 2) run_tile<RNG, 2>(a, m, it);
        else run_tile<RNG, 1>(a, m, it);
    }
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(MSIM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define BCK(expr, what)                                    \
    do {                                                   \
        cudaError_t e_ = (expr);                           \
        if (e_ != cudaSuccess) return cuda_fail(e_, what); \
    } while (0)

}  // namespace
}  // namespace msim

using namespace msim;

struct msim_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t count = 0;
    uint32_t rng_kind = 0;
    float dt = 1.f;
    std::vector<uint32_t> n;       // entities per instance
    std::vector<uint32_t> ebase;   // first entity per instance
    std::vector<InstanceDesc> desc;
    uint64_t total = 0;
    // device
    float4* road_pos = nullptr;
    uint4* road_conn = nullptr;
    uint32_t* conn = nullptr;
    InstanceDesc* d_inst = nullptr;
    WorkItem* d_items = nullptr;
    uint32_t num_items = 0;
    uint32_t* ticket = nullptr;
    uint32_t* err = nullptr;
    float2* pos = nullptr;
    uint32_t* head = nullptr;
    uint4* rng = nullptr;
    float* speed = nullptr;
    uint32_t* slot_scratch = nullptr;  // k_init writes slot ids; the batch keeps entities in place
    std::vector<void*> allocs;
    // schedule
    msim_batch_schedule sched{};
    int sms = 1;
    int blocks_per_sm = 1;
    // graphs per tick count
    std::map<uint32_t, cudaGraphExec_t> graphs;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    uint64_t launches = 0;
};

namespace {

template <typename T>
int balloc(msim_batch* b, T** p, size_t count) {
    void* raw = nullptr;
    if (!device_malloc(&raw, std::max<size_t>(count, 1) * sizeof(T)))
        return fail(MSIM_ERR_NOMEM, "device allocation failed in the batch");
    b->allocs.push_back(raw);
    *p = static_cast<T*>(raw);
    return MSIM_OK;
}

void drop_graphs(msim_batch* b) {
    for (auto& kv : b->graphs) cudaGraphExecDestroy(kv.second);
    b->graphs.clear();
}

void free_batch(msim_batch* b) {
    drop_graphs(b);
    for (void* p : b->allocs) cudaFree(p);
    b->allocs.clear();
    if (b->t0) cudaEventDestroy(b->t0);
    if (b->t1) cudaEventDestroy(b->t1);
    if (b->stream) cudaStreamDestroy(b->stream);
}

uint32_t class_of(const msim_batch_schedule& s, uint32_t n) {
    uint32_t c = 0;
    while (c + 1 < s.num_classes && n >= s.class_min_entities[c + 1]) c++;
    return c;
}

// Work list: every instance cut into tiles of its class's size, largest tiles first.
std::vector<WorkItem> make_items(const msim_batch* b, const msim_batch_schedule& s, int only_class) {
    std::vector<WorkItem> items;
    for (uint32_t i = 0; i < b->count; i++) {
        uint32_t c = class_of(s, b->n[i]);
        if (only_class >= 0 && (int)c != only_class) continue;
        uint32_t tile = std::max<uint32_t>(s.tile_entities[c], 1u);
        for (uint32_t off = 0; off < b->n[i]; off += tile)
            items.push_back(WorkItem{i, b->ebase[i] + off, std::min(tile, b->n[i] - off), s.entities_per_thread[c]});
    }
    std::stable_sort(items.begin(), items.end(), [](const WorkItem& x, const WorkItem& y) { return x.count > y.count; });
    return items;
}

int check_schedule(const msim_batch_schedule& s) {
    if (s.num_classes < 1 || s.num_classes > MSIM_BATCH_MAX_CLASSES) return fail(MSIM_ERR_INVALID, "num_classes out of range");
    if (s.block_threads < 32 || s.block_threads > 1024 || s.block_threads % 32)
        return fail(MSIM_ERR_INVALID, "block_threads must be a multiple of 32 in [32, 1024]");
    for (uint32_t c = 0; c < s.num_classes; c++) {
        uint32_t e = s.entities_per_thread[c];
        if (e != 1 && e != 2 && e != 4) return fail(MSIM_ERR_INVALID, "entities_per_thread must be 1, 2 or 4");
        if (s.tile_entities[c] == 0) return fail(MSIM_ERR_INVALID, "tile_entities must be > 0");
        if (c && s.class_min_entities[c] <= s.class_min_entities[c - 1])
            return fail(MSIM_ERR_INVALID, "class_min_entities must increase");
    }
    return MSIM_OK;
}

int upload_items(msim_batch* b, const std::vector<WorkItem>& items) {
    if (items.size() > b->num_items || !b->d_items) {
        if (b->d_items) {
            cudaFree(b->d_items);
            b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), (void*)b->d_items));
            b->d_items = nullptr;
        }
        int rc = balloc(b, &b->d_items, items.size());
        if (rc != MSIM_OK) return rc;
    }
    b->num_items = (uint32_t)items.size();
    if (!items.empty())
        BCK(cudaMemcpy(b->d_items, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice),
            "upload work items");
    drop_graphs(b);
    return MSIM_OK;
}

// The kernel instantiation for a schedule: RNG and its largest entities per thread.
using BatchKernel = void (*)(BatchArgs);
BatchKernel batch_kernel(uint32_t rng_kind, const msim_batch_schedule& s) {
    uint32_t emax = 1;
    for (uint32_t c = 0; c < s.num_classes && c < MSIM_BATCH_MAX_CLASSES; c++)
        emax = std::max(emax, s.entities_per_thread[c]);
    if (rng_kind == 1) return emax >= 4 ? k_batch_step<1, 4> : emax == 2 ? k_batch_step<1, 2> : k_batch_step<1, 1>;
    return emax >= 4 ? k_batch_step<0, 4> : emax == 2 ? k_batch_step<0, 2> : k_batch_step<0, 1>;
}

int occupancy(msim_batch* b, uint32_t threads) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel(b->rng_kind, b->sched), (int)threads, 0);
    return std::max(per_sm, 1);
}

BatchArgs args_of(msim_batch* b, uint32_t ticks) {
    BatchArgs a;
    a.road_pos = b->road_pos;
    a.road_conn = b->road_conn;
    a.conn = b->conn;
    a.inst = b->d_inst;
    a.items = b->d_items;
    a.num_items = b->num_items;
    a.ticket = b->ticket;
    a.pos = b->pos;
    a.head = b->head;
    a.rng = b->rng;
    a.speed = b->speed;
    a.dt = b->dt;
    a.ticks = ticks;
    a.err = b->err;
    return a;
}

cudaError_t enqueue(msim_batch* b, uint32_t ticks) {
    cudaError_t e = cudaMemsetAsync(b->ticket, 0, sizeof(uint32_t), b->stream);
    if (e != cudaSuccess) return e;
    const uint32_t threads = b->sched.block_threads;
    const int grid = b->sms * occupancy(b, threads);
    BatchArgs a = args_of(b, ticks);
    batch_kernel(b->rng_kind, b->sched)<<<grid, threads, 0, b->stream>>>(a);
    return cudaGetLastError();
}

int run_ticks(msim_batch* b, uint32_t ticks, bool use_graph) {
    if (!use_graph) {
        BCK(enqueue(b, ticks), "k_batch_step");
        b->launches++;
        return MSIM_OK;
    }
    auto it = b->graphs.find(ticks);
    if (it == b->graphs.end()) {
        cudaGraph_t g = nullptr;
        BCK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
        cudaError_t e = enqueue(b, ticks);
        cudaError_t e2 = cudaStreamEndCapture(b->stream, &g);
        if (e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return cuda_fail(e, "capture k_batch_step");
        }
        BCK(e2, "cudaStreamEndCapture");
        cudaGraphExec_t ex = nullptr;
        e = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        BCK(e, "cudaGraphInstantiate");
        it = b->graphs.emplace(ticks, ex).first;
    }
    BCK(cudaGraphLaunch(it->second, b->stream), "cudaGraphLaunch");
    b->launches++;
    return MSIM_OK;
}

int sync_batch(msim_batch* b) {
    BCK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    uint32_t h = 0;
    BCK(cudaMemcpy(&h, b->err, sizeof(h), cudaMemcpyDeviceToHost), "read device status");
    if (h) {
        BCK(cudaMemset(b->err, 0, sizeof(uint32_t)), "clear device status");
        return fail(MSIM_ERR_OOB, "a device-side index check failed in the batch");
    }
    return MSIM_OK;
}

}  // namespace

extern "C" {

int msim_batch_default_schedule(msim_batch_schedule* s) {
    if (!s) return fail(MSIM_ERR_INVALID, "schedule is NULL");
    std::memset(s, 0, sizeof(*s));
    s->block_threads = 256;
    s->num_classes = 3;
    const uint32_t mins[3] = {0u, 8192u, 65536u};
    for (int c = 0; c < 3; c++) {
        s->class_min_entities[c] = mins[c];
        s->entities_per_thread[c] = 1;
        s->tile_entities[c] = 4096;
    }
    return MSIM_OK;
}

int msim_batch_create(const msim_map* maps, const uint32_t* num_entities, uint32_t count, uint32_t rng_kind, float dt,
                      msim_batch** out) {
    if (!out) return fail(MSIM_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!maps || !num_entities || count == 0) return fail(MSIM_ERR_INVALID, "need at least one instance");
    if (rng_kind > 1) return fail(MSIM_ERR_INVALID, "unknown rng_kind");
    if (!(dt > 0.f) || !std::isfinite(dt)) return fail(MSIM_ERR_INVALID, "dt must be positive and finite");
    uint64_t total = 0, roads = 0, conns = 0;
    for (uint32_t i = 0; i < count; i++) {
        int rc = validate_map(maps[i]);
        if (rc != MSIM_OK) return fail(rc, "instance " + std::to_string(i) + ": " + msim_last_error());
        total += num_entities[i];
        roads += maps[i].num_roads;
        conns += maps[i].num_connections + 1ull;
    }
    if (total >= (1ull << 31) || roads >= (1ull << 32) || conns >= (1ull << 32))
        return fail(MSIM_ERR_INVALID, "batch too large for 32-bit indexing");
    msim_batch* b = new (std::nothrow) msim_batch();
    if (!b) return fail(MSIM_ERR_NOMEM, "out of host memory");
    auto bail = [&](int code) {
        free_batch(b);
        delete b;
        return code;
    };
    cudaGetDevice(&b->device);
    b->count = count;
    b->rng_kind = rng_kind;
    b->dt = dt;
    b->total = total;
    b->n.assign(num_entities, num_entities + count);
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(e, "cudaStreamCreate"));
    if (cudaEventCreate(&b->t0) != cudaSuccess || cudaEventCreate(&b->t1) != cudaSuccess)
        return bail(fail(MSIM_ERR_CUDA, "cudaEventCreate failed"));
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    // concatenated tables
    std::vector<float> rp(4 * roads);
    std::vector<uint32_t> rc(4 * roads), cl(conns);
    uint64_t ro = 0, co = 0, eo = 0;
    for (uint32_t i = 0; i < count; i++) {
        const msim_map& m = maps[i];
        b->desc.push_back(InstanceDesc{(uint32_t)ro, (uint32_t)co, m.num_roads, m.num_connections});
        b->ebase.push_back((uint32_t)eo);
        std::memcpy(&rp[4 * ro], m.road_pos, sizeof(float) * 4 * m.num_roads);
        std::memcpy(&rc[4 * ro], m.road_conn, sizeof(uint32_t) * 4 * m.num_roads);
        if (m.num_connections) std::memcpy(&cl[co], m.connections, sizeof(uint32_t) * m.num_connections);
        cl[co + m.num_connections] = m.num_connections ? m.connections[m.num_connections - 1] : 0u;
        ro += m.num_roads;
        co += m.num_connections + 1ull;
        eo += num_entities[i];
    }
    int r;
    if ((r = balloc(b, &b->road_pos, roads)) || (r = balloc(b, &b->road_conn, roads)) || (r = balloc(b, &b->conn, conns)) ||
        (r = balloc(b, &b->d_inst, count)) || (r = balloc(b, &b->ticket, 1)) || (r = balloc(b, &b->err, 1)) ||
        (r = balloc(b, &b->pos, total)) || (r = balloc(b, &b->head, total)) || (r = balloc(b, &b->rng, total)) ||
        (r = balloc(b, &b->speed, total)) || (r = balloc(b, &b->slot_scratch, total)))
        return bail(r);
    e = cudaMemcpy(b->road_pos, rp.data(), sizeof(float4) * roads, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->road_conn, rc.data(), sizeof(uint4) * roads, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->conn, cl.data(), sizeof(uint32_t) * conns, cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_inst, b->desc.data(), sizeof(InstanceDesc) * count, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(b->err, 0, sizeof(uint32_t));
    if (e != cudaSuccess) return bail(cuda_fail(e, "batch set-up"));
    msim_batch_default_schedule(&b->sched);
    r = upload_items(b, make_items(b, b->sched, -1));
    if (r != MSIM_OK) return bail(r);
    *out = b;
    return MSIM_OK;
}

int msim_batch_destroy(msim_batch* b) {
    if (!b) return MSIM_OK;
    cudaSetDevice(b->device);
    cudaStreamSynchronize(b->stream);
    free_batch(b);
    delete b;
    return MSIM_OK;
}

int msim_batch_init_entities(msim_batch* b, const msim_init* inits) {
    if (!b || !inits) return fail(MSIM_ERR_INVALID, "NULL argument");
    cudaSetDevice(b->device);
    for (uint32_t i = 0; i < b->count; i++) {
        const msim_init& in = inits[i];
        if (in.placement > 1 || !(in.speed_max >= in.speed_min)) return fail(MSIM_ERR_INVALID, "bad init for instance " + std::to_string(i));
        DeviceMap m;
        m.road_pos = b->road_pos + b->desc[i].road_base;
        m.road_conn = b->road_conn + b->desc[i].road_base;
        m.conn = b->conn + b->desc[i].conn_base;
        m.factor = nullptr;
        m.num_roads = b->desc[i].num_roads;
        m.num_conn = b->desc[i].num_conn;
        EntityState st;
        const uint32_t e0 = b->ebase[i];
        st.pos = b->pos + e0;
        st.head = b->head + e0;
        st.rng = b->rng + e0;
        st.speed = b->speed + e0;
        st.slot_id = b->slot_scratch + e0;
        BCK(launch_init_entities(b->stream, m, st, b->n[i], b->rng_kind, in.seed, in.placement, in.speed_min,
                                 in.speed_max),
            "k_init");
    }
    return sync_batch(b);
}

int msim_batch_step(msim_batch* b, uint32_t ticks) {
    msim::NvtxRange range("msim_batch_step");
    if (!b) return fail(MSIM_ERR_INVALID, "batch is NULL");
    cudaSetDevice(b->device);
    if (ticks == 0 || b->num_items == 0) return MSIM_OK;
    return run_ticks(b, ticks, true);
}

int msim_batch_sync(msim_batch* b) {
    if (!b) return fail(MSIM_ERR_INVALID, "batch is NULL");
    cudaSetDevice(b->device);
    return sync_batch(b);
}

int msim_batch_get_state(msim_batch* b, uint32_t instance, float* pos, uint32_t* heading, uint32_t* rng, float* speed) {
    if (!b) return fail(MSIM_ERR_INVALID, "batch is NULL");
    if (instance >= b->count) return fail(MSIM_ERR_INVALID, "instance out of range");
    cudaSetDevice(b->device);
    int rc = sync_batch(b);
    if (rc != MSIM_OK) return rc;
    const size_t e0 = b->ebase[instance], n = b->n[instance];
    if (pos) BCK(cudaMemcpy(pos, b->pos + e0, sizeof(float2) * n, cudaMemcpyDeviceToHost), "download pos");
    if (heading) BCK(cudaMemcpy(heading, b->head + e0, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost), "download heading");
    if (rng) BCK(cudaMemcpy(rng, b->rng + e0, sizeof(uint4) * n, cudaMemcpyDeviceToHost), "download rng");
    if (speed) BCK(cudaMemcpy(speed, b->speed + e0, sizeof(float) * n, cudaMemcpyDeviceToHost), "download speed");
    return MSIM_OK;
}

int msim_batch_set_schedule(msim_batch* b, const msim_batch_schedule* s) {
    if (!b || !s) return fail(MSIM_ERR_INVALID, "NULL argument");
    int rc = check_schedule(*s);
    if (rc != MSIM_OK) return rc;
    cudaSetDevice(b->device);
    BCK(cudaStreamSynchronize(b->stream), "cudaStreamSynchronize");
    b->sched = *s;
    return upload_items(b, make_items(b, b->sched, -1));
}

int msim_batch_get_schedule(msim_batch* b, msim_batch_schedule* s) {
    if (!b || !s) return fail(MSIM_ERR_INVALID, "NULL argument");
    *s = b->sched;
    return MSIM_OK;
}

int msim_batch_timer_begin(msim_batch* b) {
    if (!b) return fail(MSIM_ERR_INVALID, "batch is NULL");
    BCK(cudaEventRecord(b->t0, b->stream), "cudaEventRecord");
    return MSIM_OK;
}

int msim_batch_timer_end(msim_batch* b, float* ms) {
    if (!b || !ms) return fail(MSIM_ERR_INVALID, "NULL argument");
    BCK(cudaEventRecord(b->t1, b->stream), "cudaEventRecord");
    BCK(cudaEventSynchronize(b->t1), "cudaEventSynchronize");
    BCK(cudaEventElapsedTime(ms, b->t0, b->t1), "cudaEventElapsedTime");
    return MSIM_OK;
}

int msim_batch_info(msim_batch* b, uint64_t* total_entities, uint32_t* work_items, uint64_t* launches) {
    if (!b) return fail(MSIM_ERR_INVALID, "batch is NULL");
    if (total_entities) *total_entities = b->total;
    if (work_items) *work_items = b->num_items;
    if (launches) *launches = b->launches;
    return MSIM_OK;
}

// Autotuner: for each size class, time every (entities per thread, tile size)
// candidate on that class's instances alone; then time the block sizes with the
// per-class winners on the whole batch.  The state is saved before and restored
// after, so tuning does not advance the simulation.  With cache_path, a cached
// schedule for the same device, instance sizes and tick count is reused, and a
// new result is written there.
int msim_batch_tune(msim_batch* b, uint32_t ticks, const char* cache_path) {
    if (!b) return fail(MSIM_ERR_INVALID, "batch is NULL");
    if (ticks == 0) return fail(MSIM_ERR_INVALID, "ticks must be > 0");
    cudaSetDevice(b->device);
    cudaDeviceProp prop{};
    cudaGetDeviceProperties(&prop, b->device);
    std::ostringstream keyss;
    keyss << prop.name << "|" << b->rng_kind << "|" << ticks << "|" << b->count;
    uint64_t h = 1469598103934665603ull;
    for (uint32_t i = 0; i < b->count; i++) h = (h ^ b->n[i]) * 1099511628211ull;
    keyss << "|" << std::hex << h;
    const std::string key = keyss.str();
    if (cache_path) {
        std::ifstream f(cache_path);
        std::string line;
        while (std::getline(f, line)) {
            if (line.rfind(key + " ", 0) != 0) continue;
            std::istringstream is(line.substr(key.size() + 1));
            msim_batch_schedule s{};
            is >> s.block_threads >> s.num_classes;
            for (uint32_t c = 0; c < s.num_classes && c < MSIM_BATCH_MAX_CLASSES; c++)
                is >> s.class_min_entities[c] >> s.entities_per_thread[c] >> s.tile_entities[c];
            if (is && check_schedule(s) == MSIM_OK) return msim_batch_set_schedule(b, &s);
        }
    }
    // save the state
    const size_t T = b->total;
    float2* sp = nullptr;
    uint32_t* sh = nullptr;
    uint4* sr = nullptr;
    if (!device_malloc(reinterpret_cast<void**>(&sp), sizeof(float2) * T) ||
        !device_malloc(reinterpret_cast<void**>(&sh), sizeof(uint32_t) * T) ||
        !device_malloc(reinterpret_cast<void**>(&sr), sizeof(uint4) * T)) {
        cudaFree(sp);
        cudaFree(sh);
        cudaFree(sr);
        cudaGetLastError();
        return fail(MSIM_ERR_NOMEM, "no memory to save the state while tuning");
    }
    auto save = [&]() {
        cudaMemcpyAsync(sp, b->pos, sizeof(float2) * T, cudaMemcpyDeviceToDevice, b->stream);
        cudaMemcpyAsync(sh, b->head, sizeof(uint32_t) * T, cudaMemcpyDeviceToDevice, b->stream);
        cudaMemcpyAsync(sr, b->rng, sizeof(uint4) * T, cudaMemcpyDeviceToDevice, b->stream);
    };
    auto restore = [&]() {
        cudaMemcpyAsync(b->pos, sp, sizeof(float2) * T, cudaMemcpyDeviceToDevice, b->stream);
        cudaMemcpyAsync(b->head, sh, sizeof(uint32_t) * T, cudaMemcpyDeviceToDevice, b->stream);
        cudaMemcpyAsync(b->rng, sr, sizeof(uint4) * T, cudaMemcpyDeviceToDevice, b->stream);
    };
    save();
    auto time_items = [&](const msim_batch_schedule& s, int only_class, float* ms) -> int {
        b->sched = s;
        int rc = upload_items(b, make_items(b, s, only_class));
        if (rc != MSIM_OK) return rc;
        if (b->num_items == 0) {
            *ms = 0.f;
            return MSIM_OK;
        }
        restore();
        if ((rc = run_ticks(b, ticks, false)) != MSIM_OK) return rc;  // warm-up
        restore();
        BCK(cudaEventRecord(b->t0, b->stream), "cudaEventRecord");
        if ((rc = run_ticks(b, ticks, false)) != MSIM_OK) return rc;
        BCK(cudaEventRecord(b->t1, b->stream), "cudaEventRecord");
        BCK(cudaEventSynchronize(b->t1), "cudaEventSynchronize");
        BCK(cudaEventElapsedTime(ms, b->t0, b->t1), "cudaEventElapsedTime");
        return MSIM_OK;
    };
    msim_batch_schedule best;
    msim_batch_default_schedule(&best);
    int rc = MSIM_OK;
    const uint32_t epts[3] = {1, 2, 4};
    for (uint32_t c = 0; c < best.num_classes && rc == MSIM_OK; c++) {
        float best_ms = 1e30f;
        for (uint32_t e : epts) {
            for (uint32_t mult : {1u, 4u, 16u, 64u}) {
                msim_batch_schedule s = best;
                s.entities_per_thread[c] = e;
                s.tile_entities[c] = s.block_threads * e * mult;
                float ms = 0.f;
                rc = time_items(s, (int)c, &ms);
                if (rc != MSIM_OK) break;
                if (ms > 0.f && ms < best_ms) {
                    best_ms = ms;
                    best.entities_per_thread[c] = e;
                    best.tile_entities[c] = s.tile_entities[c];
                }
            }
            if (rc != MSIM_OK) break;
        }
    }
    if (rc == MSIM_OK) {
        float best_ms = 1e30f;
        msim_batch_schedule base = best;
        for (uint32_t threads : {128u, 256u, 512u}) {
            msim_batch_schedule s = base;
            s.block_threads = threads;
            for (uint32_t c = 0; c < s.num_classes; c++)  // keep the tiles' thread multiples
                s.tile_entities[c] = base.tile_entities[c] / base.block_threads * threads;
            float ms = 0.f;
            rc = time_items(s, -1, &ms);
            if (rc != MSIM_OK) break;
            if (ms < best_ms) {
                best_ms = ms;
                best = s;
            }
        }
    }
    restore();
    cudaStreamSynchronize(b->stream);
    cudaFree(sp);
    cudaFree(sh);
    cudaFree(sr);
    if (rc != MSIM_OK) return rc;
    rc = msim_batch_set_schedule(b, &best);
    if (rc == MSIM_OK && cache_path) {
        std::ofstream f(cache_path, std::ios::app);
        f << key << " " << best.block_threads << " " << best.num_classes;
        for (uint32_t c = 0; c < best.num_classes; c++)
            f << " " << best.class_min_entities[c] << " " << best.entities_per_thread[c] << " " << best.tile_entities[c];
        f << "\n";
    }
    return rc;
}

}  // extern "C"
