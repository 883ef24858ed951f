/*
 * msim.h - C ABI of the GB300 movement-sim per-tick path.
 *
 * The path: every tick each entity moves along its road toward the road end it
 * heads for; at the end it picks the next road from the connection list with its
 * own random state.  After the move, a spatial index over all entities is rebuilt
 * (sort key of the entity's tile and y band, radix sort, key-start table) and a radius
 * neighbour query runs over it.
 *
 * Conventions
 *  - Every function returns an int status (MSIM_OK on success).  On failure a
 *    message is kept per thread and returned by msim_last_error().  No C++
 *    exception crosses this ABI.
 *  - Pointers are plain host pointers unless the name says "device".  Arrays are
 *    indexed by entity id (0 .. num_entities-1) unless stated otherwise.
 *  - A context is single-threaded: callers serialise calls on one context, as the
 *    reference's worker thread does.  Separate contexts may run on separate threads.
 *  - Work is queued on the context's own CUDA stream; msim_sync() waits for it and
 *    reports device-side errors (bounded waits that gave up, indices out of range).
 *
 * Each entry point names the reference interface it replaces (file:line within
 * COM8/movement-sim).
 */
#ifndef MSIM_H
#define MSIM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
enum {
    MSIM_OK = 0,
    MSIM_ERR_INVALID = 1, /* bad argument or malformed input */
    MSIM_ERR_OOB = 2,     /* an index in map or entity data leaves its table */
    MSIM_ERR_CUDA = 3,    /* a CUDA runtime call failed */
    MSIM_ERR_TIMEOUT = 4, /* a bounded device-side wait gave up */
    MSIM_ERR_NOMEM = 5,   /* device or host allocation failed */
    MSIM_ERR_IO = 6       /* a file could not be read or written */
};

/* ---- random number generators -------------------------------------------- */
/* xorshift128 with a uvec4 state, random_move.comp:725-746 (the reference's). */
#define MSIM_RNG_XORSHIFT128 0u
/* PCG32 (PCG-XSH-RR 64/32); state = {state_lo, state_hi, inc_lo, inc_hi}. */
#define MSIM_RNG_PCG32 1u

/* Heading word: bits 0..30 = road index (Entity.hpp:44 roadIndex), bit 31 set =
 * the entity heads for the road's end, clear = for its start.  The reference
 * keeps an explicit target position (Entity.hpp:41); it is always one endpoint of
 * roads[roadIndex] (random_move.comp:787-819, Simulator.cpp:121-127). */
#define MSIM_HEADING_TO_END 0x80000000u
#define MSIM_HEADING_ROAD_MASK 0x7fffffffu

/* Entity placement for msim_init_entities. */
#define MSIM_PLACE_ROAD_START 0u       /* pos = road.start, as Simulator.cpp:121-127 */
#define MSIM_PLACE_UNIFORM_FRACTION 1u /* pos = start + u*(end-start), u in [0,1) */

/* msim_step flags */
#define MSIM_STEP_NEIGHBOURS 1u /* rebuild the index and run the neighbour query */

/* Unused neighbour slots in msim_get_neighbours output. */
#define MSIM_NO_NEIGHBOUR 0xffffffffu

/* ---- map ------------------------------------------------------------------- */
/* Road graph, caller-owned host arrays (a view).  Layout of Map.hpp:12-48:
 *   road_pos  : 4 floats per road  = start.x, start.y, end.x, end.y
 *   road_conn : 4 uint32 per road  = connIndexStart, connCountStart,
 *                                    connIndexEnd, connCountEnd
 *   connections: connectionRoadIndexList
 *   width/height: maxDistLat / maxDistLong (Map.cpp:42-52). */
typedef struct msim_map {
    uint32_t num_roads;
    uint32_t num_connections;
    const float* road_pos;
    const uint32_t* road_conn;
    const uint32_t* connections;
    float width;
    float height;
} msim_map;

/* A map owned by the library (from the JSON loader or the lattice generator). */
typedef struct msim_map_buf msim_map_buf;

/* Replaces Map::load_from_file (src/sim/Map.cpp:28-150).  Numbers are read as
 * doubles and rounded to float; roads of zero length are skipped, as Map.cpp:124-128
 * does (connection indices are kept as written).  Missing fields -> MSIM_ERR_INVALID. */
int msim_map_load_json(const char* path, msim_map_buf** out);

/* Synthetic L x L intersection lattice in the format of map/generate_map.py:234-258
 * (one connection list per node, roads ending at the node listed twice, count =
 * distinct incident roads, lists in ascending road id).  Nodes at spacing*(a,b) +
 * uniform(-jitter, jitter) + jitter, edges kept with probability keep_prob, the
 * largest component retained; every draw comes from splitmix64(seed, stream, i). */
int msim_map_generate_lattice(uint32_t side, uint64_t seed, float spacing, float jitter,
                              float keep_prob, msim_map_buf** out);

/* Fills *out with pointers into buf (valid until msim_map_free). */
int msim_map_view(const msim_map_buf* buf, msim_map* out);

/* Writes the reference JSON map format (map/generate_map.py:152-160 to_json). */
int msim_map_write_json(const msim_map* map, const char* path);

void msim_map_free(msim_map_buf* buf);

/* Checks a map the way msim_create does: every connection entry < num_roads, and
 * for each road end with count >= 2, connIndex + count <= num_connections (the
 * ranged draw of random_move.comp:743-746 can return count itself; index
 * num_connections reads a pad entry equal to the last connection). */
int msim_map_validate(const msim_map* map);

/* ---- simulation context ---------------------------------------------------- */
typedef struct msim_ctx msim_ctx;

typedef struct msim_params {
    uint32_t num_entities;    /* MAX_ENTITIES, Simulator.hpp:33 */
    uint32_t rng_kind;        /* MSIM_RNG_* */
    float dt;                 /* seconds per tick; 1.0 reproduces SPEED per dispatch */
    float radius;             /* COLLISION_RADIUS, Simulator.hpp:43 */
    uint32_t cap;             /* neighbours kept per entity, ascending id (0 = count only) */
    float cell_size;          /* spatial tile side in metres; 0 = automatic */
    uint32_t resort_interval; /* ticks between re-orderings of the entity state; 0 = automatic */
    uint32_t flags;           /* MSIM_PARAM_* bits */
} msim_params;

/* msim_params.flags: how neighbour ticks rebuild the index (same results either way).
 * By default the previous order is updated (only entries whose key changed are
 * sorted and merged back; the first neighbour tick sorts fully), and between updates
 * the index is reused: a neighbour tick queries the index built a few ticks earlier
 * with every box widened by a bound on how far any entity can have moved since
 * (ticks x max |speed| x max |road factor| x dt, plus rounding), and the index is
 * updated once that bound would pass the radius (and on the tick after
 * the entities were set, moved by the host or re-ordered).  An entity within the
 * radius of another now lay within radius + bound of it, in each coordinate, when
 * the index was built, so the results are the same.
 * FULL_SORT: always a full radix sort (e.g. entities that move far between ticks);
 * INCREMENTAL: the update (the default; kept for callers that name it);
 * NO_REUSE: update the index on every neighbour tick (host ticks included). */
#define MSIM_PARAM_FULL_SORT 1u
#define MSIM_PARAM_INCREMENTAL 2u
#define MSIM_PARAM_NO_REUSE 4u

typedef struct msim_init {
    uint64_t seed;
    uint32_t placement; /* MSIM_PLACE_* */
    float speed_min;    /* per-entity speed drawn uniformly from [speed_min, speed_max] */
    float speed_max;    /* (1.4, 1.4) with dt = 1 reproduces SPEED, random_move.comp:750 */
} msim_init;

/* No counterpart in the reference (it drives one GPU through Kompute).  Selects the
 * GPU that contexts, batches and calibrations created by the calling thread from now
 * on use (the library carries its own CUDA runtime, so the application's
 * cudaSetDevice does not reach it).  Device ids as cudaGetDeviceCount counts them;
 * default 0. */
int msim_set_device(int device);

/* Replaces Simulator::init (src/sim/Simulator.cpp:44-106): copies the map to the
 * device (with one pad connection entry), allocates entity, index and neighbour
 * buffers.  Entities start zeroed; call msim_init_entities or msim_set_entities. */
int msim_create(const msim_map* map, const msim_params* params, msim_ctx** out);

/* Replaces Simulator::~Simulator (Simulator.cpp:37-41); frees device memory. */
int msim_destroy(msim_ctx* ctx);

/* Replaces Simulator::add_entities (Simulator.cpp:114-129) and the random state of
 * Entity.cpp:44-49 with a deterministic initializer from init->seed, then builds
 * the tick-0 index (the reference's first dispatch inserts every entity into its
 * quad tree, random_move.comp:863-867). */
int msim_init_entities(msim_ctx* ctx, const msim_init* init);

/* Replaces the host->device upload of the entity buffer (Simulator.cpp:189-193).
 * pos: 2N floats, heading: N words, rng: 4N words, speed: N floats (speed may be
 * NULL for 1.4 m per tick at dt = 1).  The state stays in the caller's entity order;
 * the next neighbour tick builds the index with a full sort and the tick after it
 * re-orders the state spatially, so a caller that sets the state before every tick
 * pays no re-ordering. */
int msim_set_entities(msim_ctx* ctx, const float* pos, const uint32_t* heading,
                      const uint32_t* rng, const float* speed);

/* Per-road speed factors (num_roads floats, default 1): step = speed*factor*dt. */
int msim_set_road_factors(msim_ctx* ctx, const float* factors);

/* Replaces the per-tick pair of dispatches of Simulator::sim_tick
 * (Simulator.cpp:213-237; random_move.comp:860-879): runs `ticks` ticks.  Without
 * MSIM_STEP_NEIGHBOURS only the move runs (several ticks per launch); with it every
 * tick is move, index rebuild, neighbour query.  Asynchronous. */
int msim_step(msim_ctx* ctx, uint32_t ticks, uint32_t flags);

/* Waits for queued work (the fence wait inside kp::Sequence::eval) and reports
 * device-side errors recorded since the last call.  MSIM_ERR_TIMEOUT: a bounded
 * device wait of the spatial index gave up (see msim_set_wait_limit); the kernels
 * that read the index then skipped their work, so the entity state is intact but
 * the neighbour results of the ticks since the last successful sync are not; the
 * next neighbour tick rebuilds the index from scratch. */
int msim_sync(msim_ctx* ctx);

/* No counterpart in the reference (it has no failure detection).  Polls of a
 * look-back word by the index kernels before a wait gives up and the tick reports
 * MSIM_ERR_TIMEOUT (default 2^24, about a second; 0 restores the default). */
int msim_set_wait_limit(msim_ctx* ctx, uint32_t polls);

/* Replaces the device->host readback of the entity buffer (Simulator.cpp:248-263):
 * any pointer may be NULL.  Synchronous. */
int msim_get_state(msim_ctx* ctx, float* pos, uint32_t* heading, uint32_t* rng, float* speed);

/* Result of the last neighbour tick (replaces the collision effect of
 * random_move.comp:545-562).  count[i] = |{j != i : |dx|<=R, |dy|<=R, dist<R}|;
 * idx (N*cap words, may be NULL) holds the min(count, cap) smallest such j in
 * ascending order, the rest MSIM_NO_NEIGHBOUR.  Synchronous. */
int msim_get_neighbours(msim_ctx* ctx, uint32_t* count, uint32_t* idx);

/* One tick with the entity state on the host: the same results as
 * msim_set_entities(in_*), msim_step(ctx, 1, flags), msim_get_state(out_*) and,
 * with MSIM_STEP_NEIGHBOURS, msim_get_neighbours(out_count, out_idx) in a row.
 * Replaces one Simulator::sim_tick (Simulator.cpp:213-279: the move and collision
 * dispatches, then the entity readback of :248-263) for a caller that owns the state
 * on the host and uploads it first (Simulator.cpp:189-193).  The entities go in
 * chunks of at least 65,536 (up to 4): a chunk is moved as soon as it has arrived and
 * downloaded while later chunks still upload, so the two copy directions overlap;
 * the index and the query follow once every chunk has moved.  When the previous call
 * was also a neighbour host tick (and nothing moved or set the state since), the
 * query reads the index built from the previous state, every box widened by this
 * tick's largest displacement d (measured by the move, max(|dx|, |dy|) per entity;
 * an entity within the radius of another lay within radius + d of it, in each
 * coordinate, when that index was built), so the neighbour results are the same; the
 * index of the new state is then built after the query, while the counts download
 * and the next call's uploads run, and a device status it raises is reported by the
 * next call.  A d above the radius (large steps, host edits that move
 * entities) takes the usual order for that tick.  With page-locked host
 * buffers (msim_host_alloc) the copies run asynchronously; pageable ones work too.
 * in_speed may be NULL (1.4 m per tick at dt = 1); any output may be NULL; out_count
 * and out_idx need MSIM_STEP_NEIGHBOURS.  in_pos / out_pos (and heading, rng) may be
 * the same arrays: a chunk has been uploaded before its download writes it.  When
 * heading and rng are each one page-locked array for input and output (in place),
 * only the headings and RNG states that change (entities at a road end) are written
 * back, by the move kernel through the arrays' device mapping, and just positions
 * and counts are downloaded.  Synchronous.  A heading naming a road out of
 * range gives MSIM_ERR_OOB and keeps the context's previous state (as
 * msim_set_entities); the outputs are then undefined, and so are the input heading
 * and rng arrays when they are also the outputs (in place): chunks before the bad
 * one may already have been moved and their changed headings and RNG states written
 * back into them.  A caller that may pass bad headings and needs its arrays intact
 * passes separate output arrays. */
int msim_tick_host(msim_ctx* ctx, const float* in_pos, const uint32_t* in_heading, const uint32_t* in_rng,
                   const float* in_speed, uint32_t flags, float* out_pos, uint32_t* out_heading,
                   uint32_t* out_rng, uint32_t* out_count, uint32_t* out_idx);

/* debugData[1] of the last neighbour tick (random_move.comp:548): pairs j < i. */
int msim_get_collision_pairs(msim_ctx* ctx, uint64_t* pairs);

/* Writes n (= num_entities) 64-byte records in the layout of Entity.hpp:33-46
 * (color, randomState, pos, target, direction, roadIndex, initialized) for
 * Simulator::get_entities (Simulator.cpp:143-147).  color is green, or blue when
 * the entity had a neighbour in the last neighbour tick (random_move.comp:545-549,
 * 876); direction is recomputed from pos and target. */
int msim_export_entities_aos(msim_ctx* ctx, void* out, size_t n);

/* Reference-layout quad tree over the current positions, for
 * Simulator::get_quad_tree_nodes (Simulator.cpp:149-153).  nodes receives
 * node_capacity 64-byte records of GpuQuadTree.hpp:14-41, links (may be NULL)
 * num_entities 20-byte records of GpuQuadTree.hpp:44-62.  Entities are inserted in
 * id order with the rules of random_move.comp:309-371 (QUAD_TREE_MAX_DEPTH 8 and
 * QUAD_TREE_ENTITY_NODE_CAP 10 in Simulator.hpp:36-37).  node_capacity must hold
 * the full tree (GpuQuadTree.cpp:12-18: 21845 nodes for depth 8).  Synchronous;
 * the tree is built on the host. */
int msim_export_quad_tree(msim_ctx* ctx, uint32_t max_depth, uint32_t node_cap, void* nodes,
                          uint32_t node_capacity, void* links, uint32_t* nodes_used);

/* The same tree for positions given on the host (2n floats), no context needed. */
int msim_quad_tree_build(const float* pos, uint32_t n, float width, float height, uint32_t max_depth,
                         uint32_t node_cap, void* nodes, uint32_t node_capacity, void* links,
                         uint32_t* nodes_used);

/* No counterpart in the reference.  Neighbour sets (same predicate, cap and
 * ascending order as msim_get_neighbours) for n positions the caller holds on the
 * device, computed without allocating memory: for callers that cannot call
 * cudaMalloc at that point (it can synchronise the device and is refused during
 * stream capture; some hosts own all device memory).  Inputs/outputs are device
 * pointers: d_pos 2n floats, d_count n words, d_idx n*cap words (may be NULL when
 * cap is 0), d_status (may be NULL) one word receiving device-side error bits (0 =
 * ok).  Work is queued on `stream` (a cudaStream_t, NULL = default stream) and not
 * waited for.  n <= MSIM_NOALLOC_MAX_ENTITIES, else MSIM_ERR_INVALID; tiles are
 * capped at 512 x 512 over world_w x world_h.  All intermediates live in one
 * ~7.5 MB static device array per device, held until the process exits; every
 * call shares it, so calls whose GPU work overlaps race (serialise them).  The
 * first call on a device looks the array up (cudaGetSymbolAddress) and sets a
 * kernel attribute: make that first call before any stream capture. */
#define MSIM_NOALLOC_MAX_ENTITIES 262144u
int msim_query_neighbours_noalloc(const float* d_pos, uint32_t n, float world_w, float world_h, float radius,
                                  uint32_t cap, uint32_t* d_count, uint32_t* d_idx, uint32_t* d_status,
                                  void* stream);

/* No counterpart in the reference (its state lives only in the Kompute tensors).
 * Snapshot of the entity state by entity id (positions, headings, RNG states,
 * speeds) and the tick counter to a file, and resume from one: msim_load_state
 * checks that the file was written for the same entity count, map size and RNG,
 * then sets the state as msim_set_entities does (the next neighbour tick rebuilds
 * the index) and restores the tick counter.  A run resumed from a snapshot gives
 * the same results as the run that wrote it.  Synchronous. */
int msim_save_state(msim_ctx* ctx, const char* path);
int msim_load_state(msim_ctx* ctx, const char* path);

/* Number of ticks run since msim_create (one tick = move [+ collision]). */
int msim_get_tick(msim_ctx* ctx, uint64_t* tick);

/* Kernels this context has launched since msim_create (all kinds). */
int msim_get_launch_count(msim_ctx* ctx, uint64_t* launches);

/* Per-tick phase times, the counterpart of the per-dispatch timers of
 * Simulator::sim_tick (Simulator.cpp:213-237: update = move dispatch, collision =
 * collision dispatch).  With enable, every neighbour tick records three events on
 * the streams that run its phases (before the move, after the move, after the
 * query), which keeps the query on its own stream; msim_get_tick_times waits for
 * the last neighbour tick and returns its update time (move, plus the occasional
 * re-ordering of the state) and its collision time (index update and query). */
int msim_set_tick_timing(msim_ctx* ctx, int enable);
int msim_get_tick_times(msim_ctx* ctx, float* update_ms, float* collision_ms);

/* Device-side timing of the context's kernels (CUDA events on its stream, one pair
 * per launch; the query then runs on the context's main stream, serialised with the
 * next tick, so kernel times do not overlap). */
int msim_set_profiling(msim_ctx* ctx, int enable);
int msim_reset_kernel_stats(msim_ctx* ctx);
/* kernel: 0 .. msim_kernel_count()-1.  Synchronises the context's stream. */
int msim_get_kernel_stats(msim_ctx* ctx, uint32_t kernel, uint64_t* launches, double* total_ms);
uint32_t msim_kernel_count(void);
const char* msim_kernel_name(uint32_t kernel);
/* Index updates (full sorts and incremental updates) since the stats were reset, and
 * the entries that went through their radix passes (n per full sort, the entries
 * whose key changed per incremental update): the sort's work per tick.
 * Synchronises the context's stream. */
int msim_get_sort_stats(msim_ctx* ctx, uint64_t* index_updates, uint64_t* sorted_entries);
/* msim_tick_host calls since the stats were reset, those whose query read the
 * previous state's index with widened boxes, and the largest displacement measured by
 * the last call that measured one (any pointer may be NULL; reset with the kernel
 * stats). */
int msim_get_host_tick_stats(msim_ctx* ctx, uint64_t* host_ticks, uint64_t* skin_queries, float* last_displacement);

/* Events on the context's stream around a region of queued work (bench timing). */
int msim_timer_begin(msim_ctx* ctx);
int msim_timer_end(msim_ctx* ctx, float* ms);

/* Page-locked host memory for copies inside timed regions. */
int msim_host_alloc(size_t bytes, void** out);
int msim_host_free(void* ptr);

/* ---- batched ensemble ------------------------------------------------------------
 * Many independent instances (own road graph and entities each) advanced by one
 * persistent kernel launch, captured once per tick count into a CUDA graph.  Move
 * ticks only (no neighbour query); every instance's result is bit-identical to a
 * single context running msim_step without MSIM_STEP_NEIGHBOURS.  No reference
 * counterpart: the reference runs one map (Simulator.cpp:44-106). */
typedef struct msim_batch msim_batch;

#define MSIM_BATCH_MAX_CLASSES 4
typedef struct msim_batch_schedule {
    uint32_t block_threads;                                 /* multiple of 32 */
    uint32_t num_classes;                                   /* size classes, 1..4 */
    uint32_t class_min_entities[MSIM_BATCH_MAX_CLASSES];    /* class c: min[c] <= n < min[c+1] */
    uint32_t entities_per_thread[MSIM_BATCH_MAX_CLASSES];   /* 1, 2 or 4 */
    uint32_t tile_entities[MSIM_BATCH_MAX_CLASSES];         /* entities per work item */
} msim_batch_schedule;

int msim_batch_default_schedule(msim_batch_schedule* schedule);
int msim_batch_create(const msim_map* maps, const uint32_t* num_entities, uint32_t count, uint32_t rng_kind,
                      float dt, msim_batch** out);
int msim_batch_destroy(msim_batch* batch);
/* One msim_init per instance (same initializer as msim_init_entities). */
int msim_batch_init_entities(msim_batch* batch, const msim_init* inits);
/* Asynchronous: `ticks` move ticks of every instance in one persistent launch. */
int msim_batch_step(msim_batch* batch, uint32_t ticks);
int msim_batch_sync(msim_batch* batch);
int msim_batch_get_state(msim_batch* batch, uint32_t instance, float* pos, uint32_t* heading, uint32_t* rng,
                         float* speed);
int msim_batch_set_schedule(msim_batch* batch, const msim_batch_schedule* schedule);
int msim_batch_get_schedule(msim_batch* batch, msim_batch_schedule* schedule);
/* Autotuner: times per size class every (entities per thread, tile) candidate, then
 * the block sizes; keeps the fastest.  The simulation state is left unchanged.
 * cache_path (may be NULL): a text file of earlier results keyed by device name,
 * RNG, tick count and instance sizes; a hit skips the timing, a new result is
 * appended. */
int msim_batch_tune(msim_batch* batch, uint32_t ticks, const char* cache_path);
int msim_batch_timer_begin(msim_batch* batch);
int msim_batch_timer_end(msim_batch* batch, float* ms);
int msim_batch_info(msim_batch* batch, uint64_t* total_entities, uint32_t* work_items, uint64_t* launches);

/* ---- differentiable density calibration ------------------------------------------
 * Forward: `ticks` move ticks of the entities from the deterministic initializer,
 * step = speed[e] * factor[road] * dt; observable D = (1/ticks) sum_t splat(p_t),
 * bilinear cell-centred weights on a grid_w x grid_h grid over the world;
 * loss = mean_g (D_g - target_g)^2.  Backward: the adjoint of the kinematic step
 * and the splat with the forward's discrete events (road-end ticks and road
 * choices) held fixed; states are checkpointed every checkpoint_interval ticks and
 * recomputed; road-factor gradients are summed by a deterministic sort-based
 * segmented reduction.  Device pointers throughout.  No reference counterpart
 * (the reference has no differentiable path). */
typedef struct msim_adj msim_adj;
typedef struct msim_adj_params {
    uint32_t num_entities;
    uint32_t rng_kind;
    float dt;
    uint32_t ticks;
    uint32_t checkpoint_interval; /* K */
    uint32_t grid_w;
    uint32_t grid_h;
    uint32_t placement;           /* MSIM_PLACE_* of the initializer */
    uint64_t seed;                /* initializer seed */
    float speed_min;              /* initializer speed range (the speeds a forward without */
    float speed_max;              /* d_speed uses) */
} msim_adj_params;

#define MSIM_ADJ_NATURAL 0u /* events from the step itself; the schedule is stored */
#define MSIM_ADJ_RECORD 1u  /* the same as NATURAL (kept as a name for callers that record) */
#define MSIM_ADJ_REPLAY 2u  /* force the stored event schedule (finite differences) */

int msim_adj_create(const msim_map* map, const msim_adj_params* params, msim_adj** out);
int msim_adj_destroy(msim_adj* adj);
/* Initial state from the initializer (host arrays, any may be NULL). */
int msim_adj_get_initial_state(msim_adj* adj, float* pos, uint32_t* heading, uint32_t* rng, float* speed);
/* d_speed (n), d_factor (num_roads), d_target (grid) may be NULL to keep the
 * previous values (speeds from the initializer, factors 1, target 0); d_density
 * (grid, may be NULL) receives D; *loss (host, may be NULL).  Synchronous. */
int msim_adj_forward(msim_adj* adj, const float* d_speed, const float* d_factor, const float* d_target,
                     float* d_density, uint32_t mode, double* loss);
/* Gradients of the last forward's loss (device outputs, either may be NULL). */
int msim_adj_backward(msim_adj* adj, float* d_grad_speed, float* d_grad_factor);
/* The same gradients as accumulated (double), to host arrays. */
int msim_adj_get_gradients_f64(msim_adj* adj, double* grad_speed, double* grad_factor);
/* Event schedule of the last natural forward: one bit per entity and tick (bit
 * (t-1) % 32 of word (t-1) / 32 set when the entity reaches its road end at tick t),
 * ceil(ticks/32) words per entity. */
int msim_adj_get_schedule(msim_adj* adj, uint32_t* words);
int msim_adj_timer_begin(msim_adj* adj);
int msim_adj_timer_end(msim_adj* adj, float* ms);
/* Device time (ms, CUDA events) of the last forward and backward phases:
 * ms[0] forward kernel, ms[1] loss, ms[2] backward segment sweeps (all segments),
 * ms[3] road-gradient sort and sums. */
int msim_adj_phase_times(msim_adj* adj, float ms[4]);

/* Resolved configuration of a context (for reports). */
typedef struct msim_info {
    uint32_t num_entities;
    uint32_t num_roads;
    uint32_t num_connections;
    uint32_t tiles_x;
    uint32_t tiles_y;
    uint32_t key_bits;
    uint32_t sort_passes;
    uint32_t resort_interval;
    float cell_size;
    uint32_t cap;
    uint64_t device_bytes;
} msim_info;
int msim_get_info(msim_ctx* ctx, msim_info* out);

const char* msim_last_error(void);
const char* msim_version(void);

#ifdef __cplusplus
}
#endif

#endif /* MSIM_H */
