// sim::Simulator: the reference's C++ simulator API (src/sim/Simulator.hpp:26-137)
// over the msim C ABI.  The worker thread, pause/continue, TPS counters, tick
// histories, CSV log and snapshot hand-off behave as in the reference; the
// Kompute/Vulkan dispatches are replaced by msim_step on one CUDA stream.
//
// Differences from the reference, by design:
//  - the map and entity count come from a SimulatorConfig (the reference hard-codes
//    a path, Simulator.cpp:55, and MAX_ENTITIES, Simulator.hpp:33);
//  - entity random states come from a seed (Entity.cpp:44-49 uses std::random_device);
//  - snapshots are handed between the worker and readers under a mutex (the
//    reference moves the shared_ptr without one, Simulator.cpp:143-153).
#pragma once

#include <chrono>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <filesystem>
#include <fstream>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "msim.h"

namespace sim {

// ---- POD layouts (Entity.hpp:6-46, Map.hpp:12-25, GpuQuadTree.hpp:7-62) ----------
struct Vec2 {
    float x{0};
    float y{0};
};
struct Vec4U {
    uint32_t x{0}, y{0}, z{0}, w{0};
};
struct Rgba {
    float r{0}, g{0}, b{0}, a{0};
};
struct alignas(16) Entity {
    Rgba color{1.0f, 0.0f, 0.0f, 1.0f};
    Vec4U randomState{};
    Vec2 pos{};
    Vec2 target{};
    Vec2 direction{};
    uint32_t roadIndex{0};
    uint32_t initialized{0};
};
static_assert(sizeof(Entity) == 64, "Entity must keep the 64-byte reference layout");

struct Coordinate {
    Vec2 pos{};
    uint32_t connectedIndex{0};
    uint32_t connectedCount{0};
};
struct Road {
    Coordinate start;
    Coordinate end;
};
static_assert(sizeof(Road) == 32, "Road must keep the 32-byte reference layout");

namespace gpu_quad_tree {
enum class NextType : uint32_t { INVALID = 0, NODE = 1, ENTITY = 2 };
struct Node {
    int32_t acquireLock{0};
    int32_t writeLock{0};
    int32_t readerLock{0};
    float offsetX{0};
    float offsetY{0};
    float width{0};
    float height{0};
    NextType contentType{NextType::INVALID};
    uint32_t entityCount{0};
    uint32_t first{0};
    uint32_t prevNodeIndex{0};
    uint32_t nextTL{0};
    uint32_t nextTR{0};
    uint32_t nextBL{0};
    uint32_t nextBR{0};
    uint32_t padding{0};
};
static_assert(sizeof(Node) == 64, "Node must keep the 64-byte reference layout");
struct Entity {
    uint32_t nodeIndex{0};
    NextType typeNext{NextType::INVALID};
    uint32_t next{0};
    NextType typePrev{NextType::INVALID};
    uint32_t prev{0};
};
static_assert(sizeof(Entity) == 20, "quad-tree entity link must be 20 bytes");
void init_node_zero(Node& node, float worldSizeX, float worldSizeY);
size_t calc_node_count(size_t maxDepth);
}  // namespace gpu_quad_tree

// ---- map (Map.hpp:34-48) --------------------------------------------------------
class Map {
   public:
    float width{0};
    float height{0};
    std::vector<Road> roads;
    std::vector<uint32_t> connections;

    static std::shared_ptr<Map> load_from_file(const std::filesystem::path& path);
    static std::shared_ptr<Map> lattice(uint32_t side, uint64_t seed, float spacing = 50.f, float jitter = 10.f,
                                        float keep_prob = 0.9f);
    msim_map view() const;  // valid while this Map lives
};

// ---- tick metrics (utils/TickRate.hpp, utils/TickDurationHistory.hpp) ------------
namespace utils {
class TickRate {
   public:
    void tick();
    double get_ticks() const;

   private:
    std::chrono::steady_clock::time_point last_ = std::chrono::steady_clock::now();
    std::chrono::nanoseconds window_{0};
    double count_{0};
    double ticks_{0};
};

class TickDurationHistory {
   public:
    static constexpr size_t MAX_TIMES = 100;
    void add_time(const std::chrono::nanoseconds& time);
    std::chrono::nanoseconds get_avg_time() const;
    std::string get_avg_time_str() const;

   private:
    mutable std::mutex mu_;
    std::vector<std::chrono::nanoseconds> times_;
    size_t next_{0};
};
}  // namespace utils

// ---- simulator ----------------------------------------------------------------------
enum class SimulatorState { STOPPED, RUNNING, JOINING };

constexpr size_t MAX_ENTITIES = 1000000;           // Simulator.hpp:33
constexpr size_t QUAD_TREE_MAX_DEPTH = 8;          // Simulator.hpp:36
constexpr size_t QUAD_TREE_ENTITY_NODE_CAP = 10;   // Simulator.hpp:37
constexpr float COLLISION_RADIUS = 10;             // Simulator.hpp:43

struct SimulatorConfig {
    std::filesystem::path map_path;    // reference JSON map; empty -> lattice
    uint32_t lattice_side = 256;       // used when map_path is empty
    uint64_t seed = 20261203;
    size_t num_entities = MAX_ENTITIES;
    uint32_t rng_kind = MSIM_RNG_XORSHIFT128;
    float dt = 1.0f;                   // 1.0: one SPEED step per tick (random_move.comp:750)
    float speed_min = 1.4f;
    float speed_max = 1.4f;
    uint32_t placement = MSIM_PLACE_ROAD_START;
    float collision_radius = COLLISION_RADIUS;
    uint32_t neighbour_cap = 64;
    std::filesystem::path log_csv_path;  // empty -> "<num_entities>.csv" (Simulator.cpp:337-340)
    // Per-kernel device times (msim_get_kernel_stats) cost an event pair per launch and
    // serialise the query with the next tick; the update / collision histories come
    // from per-tick phase events (msim_set_tick_timing) either way.
    bool kernel_stats = false;
};

class Simulator {
   public:
    explicit Simulator(SimulatorConfig config = {});
    ~Simulator();
    Simulator(Simulator&&) = delete;
    Simulator(const Simulator&) = delete;
    Simulator& operator=(Simulator&&) = delete;
    Simulator& operator=(const Simulator&) = delete;

    void init();

    // Configuration used by get_instance() on first use.
    static void configure(const SimulatorConfig& config);
    static std::shared_ptr<Simulator>& get_instance();

    [[nodiscard]] SimulatorState get_state() const;
    void start_worker();
    void stop_worker();

    void continue_simulation();
    void pause_simulation();
    [[nodiscard]] bool is_simulating() const;
    [[nodiscard]] const utils::TickRate& get_tps() const;
    [[nodiscard]] const utils::TickDurationHistory& get_tps_history() const;
    [[nodiscard]] const utils::TickDurationHistory& get_update_tick_history() const;
    [[nodiscard]] const utils::TickDurationHistory& get_collision_detection_tick_history() const;
    // Takes the latest snapshot (nullptr until the worker has produced one since the
    // last call); the next tick makes a new one, as Simulator.cpp:143-147, 248-263.
    std::shared_ptr<std::vector<Entity>> get_entities();
    std::shared_ptr<std::vector<gpu_quad_tree::Node>> get_quad_tree_nodes();
    [[nodiscard]] const std::shared_ptr<Map> get_map() const;
    [[nodiscard]] bool is_initialized() const;

    // Additions: one synchronous tick without the worker; counters of the last tick.
    void tick_once();
    [[nodiscard]] uint64_t get_tick() const;
    [[nodiscard]] uint64_t get_collision_pairs() const;
    [[nodiscard]] msim_ctx* context() const { return ctx_; }

   private:
    void sim_worker();
    void sim_tick();
    void write_log_csv_file(uint64_t tick, std::chrono::nanoseconds update, std::chrono::nanoseconds collision,
                            std::chrono::nanoseconds all);

    SimulatorConfig config_;
    bool initialized_{false};
    msim_ctx* ctx_{nullptr};
    std::shared_ptr<Map> map_;
    std::unique_ptr<std::ofstream> log_file_;

    std::unique_ptr<std::thread> sim_thread_;
    SimulatorState state_{SimulatorState::STOPPED};
    std::mutex wait_mutex_;
    std::condition_variable wait_cv_;
    bool simulating_{false};

    utils::TickDurationHistory tps_history_;
    utils::TickRate tps_;
    utils::TickDurationHistory update_history_;
    utils::TickDurationHistory collision_history_;

    mutable std::mutex snapshot_mutex_;
    std::shared_ptr<std::vector<Entity>> entities_;
    std::shared_ptr<std::vector<gpu_quad_tree::Node>> quad_tree_nodes_;
    bool want_entities_{true};
    bool want_nodes_{true};
    uint64_t collision_pairs_{0};
};

}  // namespace sim
