// sim::Simulator façade over the msim C ABI (see include/msim_simulator.hpp).
// Worker/tick structure follows src/sim/Simulator.cpp:159-279; the two Kompute
// dispatches per tick become one msim_step(ctx, 1, MSIM_STEP_NEIGHBOURS).
#include "msim_simulator.hpp"

#include "msim_internal.h"

#include <cstdio>
#include <ctime>
#include <iostream>
#include <stdexcept>

namespace sim {

namespace {
void check(int rc, const char* what) {
    if (rc != MSIM_OK) throw std::runtime_error(std::string(what) + ": " + msim_last_error());
}

std::shared_ptr<Map> from_buf(msim_map_buf* buf) {
    msim_map v{};
    int rc = msim_map_view(buf, &v);
    if (rc != MSIM_OK) {
        msim_map_free(buf);
        check(rc, "msim_map_view");
    }
    auto m = std::make_shared<Map>();
    m->width = v.width;
    m->height = v.height;
    m->roads.resize(v.num_roads);
    for (uint32_t r = 0; r < v.num_roads; r++) {
        const float* p = v.road_pos + 4ull * r;
        const uint32_t* c = v.road_conn + 4ull * r;
        m->roads[r] = Road{Coordinate{Vec2{p[0], p[1]}, c[0], c[1]}, Coordinate{Vec2{p[2], p[3]}, c[2], c[3]}};
    }
    m->connections.assign(v.connections, v.connections + v.num_connections);
    msim_map_free(buf);
    return m;
}

SimulatorConfig& instance_config() {
    static SimulatorConfig cfg;
    return cfg;
}
}  // namespace

// ---- gpu_quad_tree ---------------------------------------------------------------
namespace gpu_quad_tree {
void init_node_zero(Node& node, float worldSizeX, float worldSizeY) {
    node.width = worldSizeX;
    node.height = worldSizeY;
    node.contentType = NextType::ENTITY;
}
size_t calc_node_count(size_t maxDepth) {
    size_t total = 0, level = 1;
    for (size_t d = 0; d < maxDepth; d++, level *= 4) total += level;
    return total;
}
}  // namespace gpu_quad_tree

// ---- Map ------------------------------------------------------------------------------
std::shared_ptr<Map> Map::load_from_file(const std::filesystem::path& path) {
    msim_map_buf* buf = nullptr;
    check(msim_map_load_json(path.string().c_str(), &buf), "msim_map_load_json");
    return from_buf(buf);
}

std::shared_ptr<Map> Map::lattice(uint32_t side, uint64_t seed, float spacing, float jitter, float keep_prob) {
    msim_map_buf* buf = nullptr;
    check(msim_map_generate_lattice(side, seed, spacing, jitter, keep_prob, &buf), "msim_map_generate_lattice");
    return from_buf(buf);
}

msim_map Map::view() const {
    static_assert(sizeof(Road) == 8 * sizeof(float), "Road is {pos, idx, cnt} x 2");
    msim_map v{};
    v.num_roads = static_cast<uint32_t>(roads.size());
    v.num_connections = static_cast<uint32_t>(connections.size());
    // Road interleaves positions and connection info; the ABI wants them apart, so
    // keep split copies alive in thread-local storage for the duration of the call.
    thread_local std::vector<float> pos;
    thread_local std::vector<uint32_t> conn;
    pos.resize(4 * roads.size());
    conn.resize(4 * roads.size());
    for (size_t r = 0; r < roads.size(); r++) {
        const Road& rd = roads[r];
        pos[4 * r + 0] = rd.start.pos.x;
        pos[4 * r + 1] = rd.start.pos.y;
        pos[4 * r + 2] = rd.end.pos.x;
        pos[4 * r + 3] = rd.end.pos.y;
        conn[4 * r + 0] = rd.start.connectedIndex;
        conn[4 * r + 1] = rd.start.connectedCount;
        conn[4 * r + 2] = rd.end.connectedIndex;
        conn[4 * r + 3] = rd.end.connectedCount;
    }
    v.road_pos = pos.data();
    v.road_conn = conn.data();
    v.connections = connections.data();
    v.width = width;
    v.height = height;
    return v;
}

// ---- utils ------------------------------------------------------------------------------
namespace utils {
// Ticks per second over one-second windows, scaled to exactly one second
// (TickRate.cpp:4-17).
void TickRate::tick() {
    auto now = std::chrono::steady_clock::now();
    window_ += std::chrono::duration_cast<std::chrono::nanoseconds>(now - last_);
    last_ = now;
    count_ += 1.0;
    if (window_ >= std::chrono::seconds(1)) {
        double scale = 1e9 / static_cast<double>(window_.count());
        ticks_ = count_ * scale;
        count_ -= ticks_;
        window_ -= std::chrono::seconds(1);
    }
}
double TickRate::get_ticks() const { return ticks_; }

// Moving window of the last MAX_TIMES durations (TickDurationHistory.cpp:9-32).
void TickDurationHistory::add_time(const std::chrono::nanoseconds& time) {
    std::lock_guard<std::mutex> lk(mu_);
    if (times_.size() < MAX_TIMES) {
        times_.push_back(time);
        return;
    }
    times_[next_] = time;
    next_ = (next_ + 1) % MAX_TIMES;
}
std::chrono::nanoseconds TickDurationHistory::get_avg_time() const {
    std::lock_guard<std::mutex> lk(mu_);
    if (times_.empty()) return std::chrono::nanoseconds(0);
    long long sum = 0;
    for (auto t : times_) sum += t.count();
    return std::chrono::nanoseconds(sum / static_cast<long long>(times_.size()));
}
std::string TickDurationHistory::get_avg_time_str() const {
    double t = static_cast<double>(get_avg_time().count());
    const char* unit = "ns";
    if (t >= 1e9) {
        t /= 1e9;
        unit = "s";
    } else if (t >= 1e6) {
        t /= 1e6;
        unit = "ms";
    } else if (t >= 1e3) {
        t /= 1e3;
        unit = "us";
    }
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.2f%s", t, unit);
    return buf;
}
}  // namespace utils

// ---- Simulator --------------------------------------------------------------------------
Simulator::Simulator(SimulatorConfig config) : config_(std::move(config)) {
    std::filesystem::path p = config_.log_csv_path.empty()
                                  ? std::filesystem::path(std::to_string(config_.num_entities) + ".csv")
                                  : config_.log_csv_path;
    log_file_ = std::make_unique<std::ofstream>(p, std::ios::out | std::ios::app);
}

Simulator::~Simulator() {
    if (state_ == SimulatorState::RUNNING) stop_worker();
    if (ctx_) msim_destroy(ctx_);
    if (log_file_) log_file_->close();
}

void Simulator::configure(const SimulatorConfig& config) { instance_config() = config; }

std::shared_ptr<Simulator>& Simulator::get_instance() {
    static std::shared_ptr<Simulator> instance = std::make_shared<Simulator>(instance_config());
    if (!instance->is_initialized()) instance->init();
    return instance;
}

void Simulator::init() {
    if (initialized_) throw std::logic_error("Simulator::init called twice");
    map_ = config_.map_path.empty() ? Map::lattice(config_.lattice_side, config_.seed)
                                    : Map::load_from_file(config_.map_path);
    msim_map view = map_->view();
    msim_params p{};
    p.num_entities = static_cast<uint32_t>(config_.num_entities);
    p.rng_kind = config_.rng_kind;
    p.dt = config_.dt;
    p.radius = config_.collision_radius;
    p.cap = config_.neighbour_cap;
    check(msim_create(&view, &p, &ctx_), "msim_create");
    msim_init ini{config_.seed, config_.placement, config_.speed_min, config_.speed_max};
    check(msim_init_entities(ctx_, &ini), "msim_init_entities");
    check(msim_set_tick_timing(ctx_, 1), "msim_set_tick_timing");
    if (config_.kernel_stats) check(msim_set_profiling(ctx_, 1), "msim_set_profiling");
    auto ents = std::make_shared<std::vector<Entity>>(config_.num_entities);
    check(msim_export_entities_aos(ctx_, ents->data(), ents->size()), "msim_export_entities_aos");
    {
        std::lock_guard<std::mutex> lk(snapshot_mutex_);
        entities_ = ents;
        want_entities_ = false;
    }
    initialized_ = true;
}

bool Simulator::is_initialized() const { return initialized_; }
SimulatorState Simulator::get_state() const { return state_; }

std::shared_ptr<std::vector<Entity>> Simulator::get_entities() {
    std::lock_guard<std::mutex> lk(snapshot_mutex_);
    want_entities_ = true;
    return std::move(entities_);
}

std::shared_ptr<std::vector<gpu_quad_tree::Node>> Simulator::get_quad_tree_nodes() {
    std::lock_guard<std::mutex> lk(snapshot_mutex_);
    want_nodes_ = true;
    return std::move(quad_tree_nodes_);
}

const std::shared_ptr<Map> Simulator::get_map() const { return map_; }

void Simulator::start_worker() {
    if (!initialized_) throw std::logic_error("Simulator not initialized");
    if (state_ != SimulatorState::STOPPED || sim_thread_) throw std::logic_error("worker already running");
    state_ = SimulatorState::RUNNING;
    sim_thread_ = std::make_unique<std::thread>(&Simulator::sim_worker, this);
}

void Simulator::stop_worker() {
    if (state_ != SimulatorState::RUNNING || !sim_thread_) throw std::logic_error("worker not running");
    {
        std::lock_guard<std::mutex> lk(wait_mutex_);
        state_ = SimulatorState::JOINING;
    }
    wait_cv_.notify_all();
    if (sim_thread_->joinable()) sim_thread_->join();
    sim_thread_ = nullptr;
    state_ = SimulatorState::STOPPED;
}

void Simulator::continue_simulation() {
    {
        std::lock_guard<std::mutex> lk(wait_mutex_);
        if (simulating_) return;
        simulating_ = true;
    }
    wait_cv_.notify_all();
}

void Simulator::pause_simulation() {
    {
        std::lock_guard<std::mutex> lk(wait_mutex_);
        if (!simulating_) return;
        simulating_ = false;
    }
    wait_cv_.notify_all();
}

bool Simulator::is_simulating() const { return simulating_; }
const utils::TickRate& Simulator::get_tps() const { return tps_; }
const utils::TickDurationHistory& Simulator::get_tps_history() const { return tps_history_; }
const utils::TickDurationHistory& Simulator::get_update_tick_history() const { return update_history_; }
const utils::TickDurationHistory& Simulator::get_collision_detection_tick_history() const {
    return collision_history_;
}

void Simulator::sim_worker() {  // Simulator.cpp:185-211
    std::unique_lock<std::mutex> lk(wait_mutex_);
    while (state_ == SimulatorState::RUNNING) {
        if (!simulating_) wait_cv_.wait(lk);
        if (!simulating_ || state_ != SimulatorState::RUNNING) continue;
        lk.unlock();
        sim_tick();
        lk.lock();
    }
}

void Simulator::tick_once() {
    if (!initialized_) throw std::logic_error("Simulator not initialized");
    sim_tick();
}

uint64_t Simulator::get_tick() const {
    uint64_t t = 0;
    if (ctx_) msim_get_tick(ctx_, &t);
    return t;
}

uint64_t Simulator::get_collision_pairs() const {
    std::lock_guard<std::mutex> lk(snapshot_mutex_);
    return collision_pairs_;
}

void Simulator::sim_tick() {  // Simulator.cpp:213-279
    msim::NvtxRange range("sim::Simulator::sim_tick");
    auto t0 = std::chrono::steady_clock::now();
    check(msim_step(ctx_, 1, MSIM_STEP_NEIGHBOURS), "msim_step");
    check(msim_sync(ctx_), "msim_sync");
    auto all = std::chrono::steady_clock::now() - t0;

    // device time of the update (move, re-ordering) and collision (index + query)
    // phases of the tick, from the phase events on the context's two streams
    float update_ms = 0.f, collision_ms = 0.f;
    check(msim_get_tick_times(ctx_, &update_ms, &collision_ms), "msim_get_tick_times");
    auto upd = std::chrono::nanoseconds(static_cast<long long>(update_ms * 1e6));
    auto col = std::chrono::nanoseconds(static_cast<long long>(collision_ms * 1e6));
    update_history_.add_time(upd);
    collision_history_.add_time(col);
    uint64_t tick = 0;
    msim_get_tick(ctx_, &tick);
    write_log_csv_file(tick, upd, col, std::chrono::duration_cast<std::chrono::nanoseconds>(all));

    uint64_t pairs = 0;
    check(msim_get_collision_pairs(ctx_, &pairs), "msim_get_collision_pairs");
    bool want_e, want_n;
    {
        std::lock_guard<std::mutex> lk(snapshot_mutex_);
        collision_pairs_ = pairs;
        want_e = want_entities_;
        want_n = want_nodes_;
    }
    if (want_e) {
        auto ents = std::make_shared<std::vector<Entity>>(config_.num_entities);
        check(msim_export_entities_aos(ctx_, ents->data(), ents->size()), "msim_export_entities_aos");
        std::lock_guard<std::mutex> lk(snapshot_mutex_);
        entities_ = ents;
        want_entities_ = false;
    }
    if (want_n) {
        auto nodes = std::make_shared<std::vector<gpu_quad_tree::Node>>(
            gpu_quad_tree::calc_node_count(QUAD_TREE_MAX_DEPTH));
        uint32_t used = 0;
        check(msim_export_quad_tree(ctx_, QUAD_TREE_MAX_DEPTH, QUAD_TREE_ENTITY_NODE_CAP, nodes->data(),
                                    static_cast<uint32_t>(nodes->size()), nullptr, &used),
              "msim_export_quad_tree");
        std::lock_guard<std::mutex> lk(snapshot_mutex_);
        quad_tree_nodes_ = nodes;
        want_nodes_ = false;
    }
    tps_history_.add_time(std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0));
    tps_.tick();
}

// "<hh:mm:ss.mmm>;<tick>;<secUpdate>;<secCollision>;<secAll>" (Simulator.cpp:389-400)
void Simulator::write_log_csv_file(uint64_t tick, std::chrono::nanoseconds update, std::chrono::nanoseconds collision,
                                   std::chrono::nanoseconds all) {
    if (!log_file_ || !log_file_->is_open()) return;
    auto now = std::chrono::system_clock::now();
    auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(now.time_since_epoch()).count();
    std::time_t secs = static_cast<std::time_t>(ms / 1000);
    std::tm tm{};
    gmtime_r(&secs, &tm);
    char stamp[32];
    std::snprintf(stamp, sizeof(stamp), "%02d:%02d:%02d.%03lld", tm.tm_hour, tm.tm_min, tm.tm_sec,
                  static_cast<long long>(ms % 1000));
    char line[160];
    std::snprintf(line, sizeof(line), "%s;%llu;%.6f;%.6f;%.6f\n", stamp, static_cast<unsigned long long>(tick),
                  update.count() / 1e9, collision.count() / 1e9, all.count() / 1e9);
    (*log_file_) << line;
    log_file_->flush();
}

}  // namespace sim
