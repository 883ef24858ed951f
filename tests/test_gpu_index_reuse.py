"""Index reuse on neighbour ticks (msim_params.flags without MSIM_PARAM_NO_REUSE):
between index updates a tick queries the index built a few ticks earlier with every
box widened by a bound on the displacement since.  Counts, id lists, pair counts and
states are compared bit for bit, every tick, with the oracle and with a context that
updates the index every tick."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(sim, ref, orc, ost, radius, cap, what):
    st, rst = sim.get_state(), ref.get_state()
    for k in ("pos", "heading", "rng"):
        assert np.array_equal(st[k].view(np.uint32), rst[k].view(np.uint32)), f"{k} differs from no-reuse {what}"
    assert np.array_equal(st["pos"].view(np.uint32), ost[0].view(np.uint32)), f"positions differ {what}"
    assert np.array_equal(st["heading"], ost[1]) and np.array_equal(st["rng"], ost[2]), f"state differs {what}"
    cnt, idx = sim.get_neighbours()
    ocnt, oidx, opairs = orc.neighbours(ost[0], radius, cap, threads=8)
    assert np.array_equal(cnt, ocnt), f"counts differ {what}"
    assert np.array_equal(idx, oidx), f"lists differ {what}"
    rcnt, ridx = ref.get_neighbours()
    assert np.array_equal(cnt, rcnt) and np.array_equal(idx, ridx)
    assert sim.collision_pairs() == opairs


@pytest.mark.parametrize("side,n,cap,rng,index", [(48, 200_000, 16, "pcg32", "auto"),
                                                  (16, 100_000, 8, "xorshift128", "auto"),
                                                  (48, 200_000, 16, "xorshift128", "full")])
def test_reuse_matches_oracle_every_tick(msim, orc, side, n, cap, rng, index):
    """(48, 200,000): tiles of about 11 m; (16, 100,000): tiles of 2 x reach, so widened
    boxes span three tiles, and about 15 neighbours per entity (beyond the eight kept
    in registers).  Calls of 1 to 5 ticks (the query of a tick overlaps the next tick),
    re-ordering every 5 ticks, move-only steps in between, then road factors up to 2
    (a larger bound, so fewer ticks reuse the index).  With incremental updates the
    moves of reusing ticks place the positions by the update's ranks; with full sorts
    (no ranks) a gather pass does."""
    road_map = msim.RoadMap.lattice(side, 7)
    rk = {"xorshift128": 0, "pcg32": 1}[rng]
    radius, dt = 2.0, 0.1
    kw = dict(rng=rng, dt=dt, radius=radius, cap=cap, resort_interval=5, index=index)
    with msim.Simulation(road_map, n, **kw) as sim, msim.Simulation(road_map, n, reuse=False, **kw) as ref:
        for s in (sim, ref):
            s.init_entities(3, placement="fraction", speed=(1.0, 1.6))
        st = sim.get_state()
        ost = [st["pos"].copy(), st["heading"].copy(), st["rng"].copy(), st["speed"].copy()]
        factor = None

        def advance(ticks):
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, ost[0], ost[1], ost[2], ost[3], rk,
                     dt, ticks, factor=factor, threads=8)

        tick = 0
        updates0 = sim.sort_stats()["index_updates"]
        for calls in ([1] * 12, [3, 2, 5, 1, 4], "move", [1] * 6, "factors", [1] * 10, [2, 3]):
            if calls == "move":  # move-only ticks: the index falls further behind
                for s in (sim, ref):
                    s.step(2)
                advance(2)
                tick += 2
                continue
            if calls == "factors":
                factor = np.random.default_rng(side).uniform(0.5, 2.0, road_map.num_roads).astype(np.float32)
                for s in (sim, ref):
                    s.set_road_factors(factor)
                continue
            for k in calls:
                for s in (sim, ref):
                    s.step(k, neighbours=True)
                advance(k)
                tick += k
                _check(sim, ref, orc, ost, radius, cap, f"at tick {tick}")
        nbr_ticks = 12 + 15 + 6 + 10 + 5
        updates = sim.sort_stats()["index_updates"] - updates0
        assert updates < nbr_ticks * 0.6, (updates, nbr_ticks)  # most ticks reused the index
        assert ref.sort_stats()["index_updates"] - updates0 >= nbr_ticks


def test_reuse_off_when_steps_are_large(msim, orc):
    """Reference mode (dt = 1, 1.4 m per tick) with a 1 m radius: the bound passes
    the radius after one tick, so every neighbour tick updates the index."""
    road_map = msim.RoadMap.lattice(32, 2)
    n = 30_000
    with msim.Simulation(road_map, n, rng="xorshift128", dt=1.0, radius=1.0, cap=8) as sim:
        sim.init_entities(5, placement="fraction", speed=(1.4, 1.4))
        st = sim.get_state()
        ost = [st["pos"].copy(), st["heading"].copy(), st["rng"].copy(), st["speed"].copy()]
        u0 = sim.sort_stats()["index_updates"]
        for t in range(6):
            sim.step(1, neighbours=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, ost[0], ost[1], ost[2], ost[3], 0,
                     1.0, 1, threads=8)
            cnt, idx = sim.get_neighbours()
            ocnt, oidx, _ = orc.neighbours(ost[0], 1.0, 8, threads=8)
            assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx), f"neighbours differ at tick {t + 1}"
        assert sim.sort_stats()["index_updates"] - u0 == 6


def test_reuse_far_from_the_map(msim, orc):
    """Entities set 50 km away from a 0.8 km map (positions with an ulp of 4 mm), in a
    cluster a few metres across, heading back to their roads: the bound's rounding
    term follows the largest coordinate, and the reused index stays exact."""
    road_map = msim.RoadMap.lattice(16, 4)
    n = 20_000
    rs = np.random.default_rng(9)
    with msim.Simulation(road_map, n, rng="pcg32", dt=0.1, radius=2.0, cap=16) as sim:
        sim.init_entities(2, placement="fraction", speed=(1.0, 1.6))
        st = sim.get_state()
        pos = (np.float32([50_000.0, -30_000.0]) + rs.uniform(-15.0, 15.0, (n, 2))).astype(np.float32)
        sim.set_entities(pos, st["heading"], st["rng"], st["speed"])
        ost = [pos.copy(), st["heading"].copy(), st["rng"].copy(), st["speed"].copy()]
        u0 = sim.sort_stats()["index_updates"]
        for t in range(30):
            sim.step(1, neighbours=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, ost[0], ost[1], ost[2], ost[3], 1,
                     0.1, 1, threads=8)
            got = sim.get_state()
            assert np.array_equal(got["pos"].view(np.uint32), ost[0].view(np.uint32)), f"positions differ at {t + 1}"
            cnt, idx = sim.get_neighbours()
            ocnt, oidx, _ = orc.neighbours(ost[0], 2.0, 16, threads=8)
            assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx), f"neighbours differ at tick {t + 1}"
        assert ocnt.sum() > n  # a crowd: the widened boxes matter
        assert sim.sort_stats()["index_updates"] - u0 < 30
