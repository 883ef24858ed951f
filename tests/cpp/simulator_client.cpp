// C++ client of the sim::Simulator façade, as the reference's UI and headless
// runner use it (src/main.cpp:20-32, SimulationWidget.cpp:89-114).  Built and
// run by tests/test_simulator_cpp.py; prints "ok" and exits 0 on success.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <thread>

#include "msim_simulator.hpp"

#define REQUIRE(c)                                                        \
    do {                                                                  \
        if (!(c)) {                                                       \
            std::fprintf(stderr, "FAILED %s at line %d\n", #c, __LINE__); \
            return 1;                                                     \
        }                                                                 \
    } while (0)

int main(int argc, char** argv) {
    sim::SimulatorConfig cfg;
    cfg.lattice_side = 48;
    cfg.num_entities = 20000;
    cfg.collision_radius = 10.0f;
    cfg.log_csv_path = argc > 1 ? argv[1] : "sim_log.csv";
    sim::Simulator::configure(cfg);
    auto& s = sim::Simulator::get_instance();
    REQUIRE(s->is_initialized());
    REQUIRE(s->get_state() == sim::SimulatorState::STOPPED);
    REQUIRE(s->get_map()->roads.size() > 3000);
    REQUIRE(sim::gpu_quad_tree::calc_node_count(8) == 21845);

    // the initial snapshot exists before any tick (Simulator.cpp:114-129)
    auto e0 = s->get_entities();
    REQUIRE(e0 && e0->size() == cfg.num_entities);
    REQUIRE((*e0)[0].initialized == 1);

    // synchronous ticks
    for (int i = 0; i < 5; i++) s->tick_once();
    REQUIRE(s->get_tick() == 5);
    auto e1 = s->get_entities();
    REQUIRE(e1 && e1->size() == cfg.num_entities);
    size_t blue = 0, moved = 0;
    for (size_t i = 0; i < e1->size(); i++) {
        const sim::Entity& a = (*e0)[i];
        const sim::Entity& b = (*e1)[i];
        if (b.color.b == 1.0f) blue++;
        if (a.pos.x != b.pos.x || a.pos.y != b.pos.y) moved++;
        REQUIRE(b.roadIndex < s->get_map()->roads.size());
    }
    REQUIRE(moved > cfg.num_entities / 2);
    REQUIRE(blue > 0);  // R = 10 m at this density gives collisions
    REQUIRE(s->get_collision_pairs() > 0);
    auto nodes = s->get_quad_tree_nodes();
    REQUIRE(nodes && nodes->size() == 21845);
    uint64_t in_leaves = 0;
    for (const auto& nd : *nodes)
        if (nd.contentType == sim::gpu_quad_tree::NextType::ENTITY) in_leaves += nd.entityCount;
    REQUIRE(in_leaves == cfg.num_entities);
    REQUIRE((*nodes)[0].contentType == sim::gpu_quad_tree::NextType::NODE);

    // worker thread with pause / continue (Simulator.cpp:155-211, 281-297)
    s->start_worker();
    REQUIRE(s->get_state() == sim::SimulatorState::RUNNING);
    s->continue_simulation();
    REQUIRE(s->is_simulating());
    std::this_thread::sleep_for(std::chrono::milliseconds(1500));
    s->pause_simulation();
    std::this_thread::sleep_for(std::chrono::milliseconds(100));
    uint64_t t_paused = s->get_tick();
    REQUIRE(t_paused > 20);
    std::this_thread::sleep_for(std::chrono::milliseconds(200));
    REQUIRE(s->get_tick() == t_paused);
    REQUIRE(s->get_tps().get_ticks() > 0.0);
    REQUIRE(s->get_tps_history().get_avg_time().count() > 0);
    REQUIRE(s->get_collision_detection_tick_history().get_avg_time().count() > 0);
    REQUIRE(s->get_update_tick_history().get_avg_time().count() > 0);
    s->stop_worker();
    REQUIRE(s->get_state() == sim::SimulatorState::STOPPED);
    auto e2 = s->get_entities();
    REQUIRE(e2 && e2->size() == cfg.num_entities);
    std::printf("ticks=%llu tps=%.1f avg=%s pairs=%llu\nok\n", (unsigned long long)s->get_tick(),
                s->get_tps().get_ticks(), s->get_tps_history().get_avg_time_str().c_str(),
                (unsigned long long)s->get_collision_pairs());
    return 0;
}
