// Headless run of the sim::Simulator façade, the way the reference's runner drives
// its simulator (src/main.cpp:20-32: get_instance, then ticks), timed: `ticks`
// synchronous tick_once() calls, each a move + collision tick followed by the
// façade's bookkeeping (phase times, CSV log line, pair counter).  Prints one JSON
// line with the tick rate and the average update / collision phase times.
//
//   simulator_ticks <lattice side> <entities> <ticks> <warm-up ticks> <log csv>
//
// The workload is the synthetic lattice with PCG32 entities, dt = 0.1 s, speeds
// U[1.0, 1.6] m/s placed at a uniform fraction along their road, radius 2 m, 64
// neighbours kept.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <exception>

#include "msim_simulator.hpp"

int main(int argc, char** argv) {
    if (argc != 6) {
        std::fprintf(stderr, "usage: %s <lattice side> <entities> <ticks> <warm-up ticks> <log csv>\n", argv[0]);
        return 2;
    }
    try {
        sim::SimulatorConfig cfg;
        cfg.lattice_side = static_cast<uint32_t>(std::strtoul(argv[1], nullptr, 10));
        cfg.num_entities = std::strtoull(argv[2], nullptr, 10);
        const long ticks = std::strtol(argv[3], nullptr, 10), warmup = std::strtol(argv[4], nullptr, 10);
        cfg.log_csv_path = argv[5];
        cfg.rng_kind = MSIM_RNG_PCG32;
        cfg.dt = 0.1f;
        cfg.speed_min = 1.0f;
        cfg.speed_max = 1.6f;
        cfg.placement = MSIM_PLACE_UNIFORM_FRACTION;
        cfg.collision_radius = 2.0f;
        cfg.neighbour_cap = 64;
        sim::Simulator s(cfg);
        s.init();
        for (long i = 0; i < warmup; i++) s.tick_once();
        const auto t0 = std::chrono::steady_clock::now();
        for (long i = 0; i < ticks; i++) s.tick_once();
        const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        std::printf(
            "{\"ticks\": %ld, \"seconds\": %.6f, \"ticks_per_s\": %.3f, \"entity_steps_per_s\": %.6e, "
            "\"ms_per_tick\": %.6f, \"avg_update_ms\": %.6f, \"avg_collision_ms\": %.6f, \"pairs\": %llu}\n",
            ticks, sec, ticks / sec, (double)cfg.num_entities * ticks / sec, 1e3 * sec / ticks,
            s.get_update_tick_history().get_avg_time().count() / 1e6,
            s.get_collision_detection_tick_history().get_avg_time().count() / 1e6,
            (unsigned long long)s.get_collision_pairs());
    } catch (const std::exception& e) {
        std::fprintf(stderr, "simulator_ticks: %s\n", e.what());
        return 1;
    }
    return 0;
}
