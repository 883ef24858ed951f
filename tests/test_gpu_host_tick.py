"""msim_tick_host: one tick with the entity state on the host (chunked upload, move,
download, then index + query), against the same tick through the separate calls
(msim_set_entities, msim_step, msim_get_state, msim_get_neighbours) and the oracle.
Everything is compared bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _same_state(a, b, what):
    assert np.array_equal(a["pos"].view(np.uint32), b["pos"].view(np.uint32)), f"positions differ {what}"
    assert np.array_equal(a["heading"], b["heading"]), f"headings differ {what}"
    assert np.array_equal(a["rng"], b["rng"]), f"RNG states differ {what}"


@pytest.mark.parametrize("n,index", [(300_000, "auto"), (300_000, "incremental"), (70_000, "incremental"),
                                     (1, "auto")])
def test_tick_host_matches_separate_calls_and_oracle(msim, orc, n, index):
    """300,000 entities go in five chunks of 65,536 (the last ragged), 70,000 in two.
    With the incremental index, host ticks after the first update the previous order."""
    road_map = msim.RoadMap.lattice(64, 9)
    kw = dict(rng="pcg32", dt=0.1, radius=2.0, cap=16)
    with msim.Simulation(road_map, n, index=index, **kw) as a, msim.Simulation(road_map, n, **kw) as b:
        a.init_entities(5, placement="fraction", speed=(1.0, 1.6))
        st = a.get_state()
        speed = st["speed"].copy()
        pos, head, rng = st["pos"].copy(), st["heading"].copy(), st["rng"].copy()
        out = {"pos": msim.PinnedBuffer((n, 2), np.float32), "heading": msim.PinnedBuffer(n, np.uint32),
               "rng": msim.PinnedBuffer((n, 4), np.uint32), "count": msim.PinnedBuffer(n, np.uint32),
               "idx": msim.PinnedBuffer((n, 16), np.uint32)}
        arrays = {k: v.array for k, v in out.items()}
        for t in range(4):
            got = a.tick_host(st, neighbours=True, out=arrays)
            b.set_entities(st["pos"], st["heading"], st["rng"], st["speed"])
            b.step(1, neighbours=True)
            ref = b.get_state()
            cnt, idx = b.get_neighbours()
            _same_state(got, ref, f"from the separate calls at tick {t + 1}")
            assert np.array_equal(got["count"], cnt) and np.array_equal(got["idx"], idx)
            # the context's own exports agree (its state may now sit in another slot order)
            _same_state(a.get_state(), ref, f"from the context after the host tick {t + 1}")
            acnt, aidx = a.get_neighbours()
            assert np.array_equal(acnt, cnt) and np.array_equal(aidx, idx)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 1, 0.1, 1,
                     threads=8)
            ocnt, oidx, _ = orc.neighbours(pos, 2.0, 16, threads=8)
            _same_state(got, {"pos": pos, "heading": head, "rng": rng}, f"from the oracle at tick {t + 1}")
            assert np.array_equal(got["count"], ocnt) and np.array_equal(got["idx"], oidx)
            st = {"pos": got["pos"].copy(), "heading": got["heading"].copy(), "rng": got["rng"].copy(),
                  "speed": speed}
        assert a.tick == 4
        assert a.collision_pairs() == int(ocnt.sum()) // 2
        for buf in out.values():
            buf.free()


@pytest.mark.parametrize("index", ["incremental", "full"])
def test_ticks_after_tick_host(msim, orc, index):
    """Regular neighbour ticks after a host tick (re-ordering on the next tick, then
    incremental or full index updates) stay equal to the oracle."""
    road_map = msim.RoadMap.lattice(40, 3)
    n = 90_000
    with msim.Simulation(road_map, n, rng="xorshift128", dt=0.1, radius=2.0, cap=8, resort_interval=4,
                         index=index) as sim:
        sim.init_entities(8, placement="fraction", speed=(1.0, 1.6))
        st = sim.get_state()
        pos, head, rng, speed = st["pos"].copy(), st["heading"].copy(), st["rng"].copy(), st["speed"].copy()
        sim.tick_host(st, neighbours=True)
        orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 0, 0.1, 1)
        for t in range(10):
            sim.step(1, neighbours=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 0, 0.1, 1)
            _same_state(sim.get_state(), {"pos": pos, "heading": head, "rng": rng}, f"at tick {t + 2}")
            cnt, idx = sim.get_neighbours()
            ocnt, oidx, _ = orc.neighbours(pos, 2.0, 8, threads=8)
            assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx), f"neighbours differ at tick {t + 2}"


def test_tick_host_move_only_default_speed(msim, orc):
    """Without MSIM_STEP_NEIGHBOURS and without speeds: SPEED = 1.4 m per tick at dt = 1
    (reference mode), no neighbour outputs."""
    road_map = msim.RoadMap.lattice(16, 2)
    n = 20_000
    with msim.Simulation(road_map, n, rng="xorshift128", dt=1.0, radius=10.0, cap=4) as sim:
        sim.init_entities(3, placement="start", speed=(1.4, 1.4))
        st = sim.get_state()
        pos, head, rng = st["pos"].copy(), st["heading"].copy(), st["rng"].copy()
        speed = np.full(n, 1.4, np.float32)
        state = {"pos": st["pos"], "heading": st["heading"], "rng": st["rng"]}
        for t in range(5):
            state = sim.tick_host(state, neighbours=False)
            assert "count" not in state
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 0, 1.0, 1)
            _same_state(state, {"pos": pos, "heading": head, "rng": rng}, f"at tick {t + 1}")
        with pytest.raises(msim.MsimError) as e:  # no neighbour tick has run
            sim.get_neighbours()
        assert e.value.code == 1


def test_tick_host_bad_heading_keeps_state(msim):
    road_map = msim.RoadMap.lattice(16, 2)
    n = 100_000
    with msim.Simulation(road_map, n, rng="pcg32", dt=0.1, radius=2.0, cap=4) as sim:
        sim.init_entities(1, placement="fraction", speed=(1.0, 1.6))
        sim.step(2, neighbours=True)
        before = sim.get_state()
        bad = {k: v.copy() for k, v in before.items()}
        bad["heading"][77_777] = road_map.num_roads  # in the second chunk
        with pytest.raises(msim.MsimError) as e:
            sim.tick_host(bad, neighbours=True)
        assert e.value.code == 2 and "77777" in str(e.value)
        after = sim.get_state()
        for k in before:
            assert np.array_equal(before[k], after[k])
        assert sim.tick == 2
        sim.step(1, neighbours=True)  # the context stays usable
        sim.sync()


def test_host_ticks_with_host_edits_and_mixed_calls(msim, orc):
    """Incremental host ticks while the host moves entities between ticks (teleports
    to other roads: many keys change at once), then regular ticks (the second
    re-orders the state), then a host tick again (a full sort, as the slots no longer
    hold entity ids)."""
    road_map = msim.RoadMap.lattice(48, 4)
    n = 150_000
    rs = np.random.default_rng(0)
    with msim.Simulation(road_map, n, rng="pcg32", dt=0.1, radius=2.0, cap=8, index="incremental") as sim:
        sim.init_entities(2, placement="fraction", speed=(1.0, 1.6))
        st = sim.get_state()
        speed = st["speed"].copy()
        state = {"pos": st["pos"].copy(), "heading": st["heading"].copy(), "rng": st["rng"].copy(), "speed": speed}
        for t in range(6):
            if t in (2, 5):  # the host teleports 20,000 entities to the start of random roads
                who = rs.choice(n, 20_000, replace=False)
                roads = rs.integers(0, road_map.num_roads, who.size)
                state["pos"][who] = road_map.road_pos[roads, :2]
                state["heading"][who] = roads.astype(np.uint32) | np.uint32(0x80000000)
            pos, head, rng = state["pos"].copy(), state["heading"].copy(), state["rng"].copy()
            if t in (3, 4):  # regular ticks in between (the second re-orders the state)
                if t == 3:
                    sim.set_entities(state["pos"], state["heading"], state["rng"], speed)
                sim.step(1, neighbours=True)
                got = sim.get_state()
                got["count"] = sim.get_neighbours(with_idx=False)[0]
            else:
                got = sim.tick_host(state, neighbours=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 1, 0.1, 1,
                     threads=8)
            _same_state(got, {"pos": pos, "heading": head, "rng": rng}, f"at tick {t + 1}")
            ocnt, _, _ = orc.neighbours(pos, 2.0, 8, threads=8, with_idx=False)
            assert np.array_equal(got["count"], ocnt), f"counts differ at tick {t + 1}"
            state = {"pos": got["pos"].copy(), "heading": got["heading"].copy(), "rng": got["rng"].copy(),
                     "speed": speed}


@pytest.mark.parametrize("pinned", [True, False])
def test_tick_host_in_place(msim, orc, pinned):
    """The same arrays as input and output: with page-locked arrays only positions are
    downloaded and the changed headings / RNG states are written into the arrays by
    the move kernel; with pageable ones everything is downloaded.  Either way the
    arrays hold the oracle's state after every tick, also when the host edits them."""
    road_map = msim.RoadMap.lattice(32, 6)
    n = 200_000
    rs = np.random.default_rng(3)
    with msim.Simulation(road_map, n, rng="xorshift128", dt=0.1, radius=2.0, cap=8, index="incremental") as sim:
        sim.init_entities(9, placement="fraction", speed=(1.0, 1.6))
        st = sim.get_state()
        bufs = {}
        if pinned:
            bufs = {"pos": msim.PinnedBuffer((n, 2), np.float32), "heading": msim.PinnedBuffer(n, np.uint32),
                    "rng": msim.PinnedBuffer((n, 4), np.uint32), "count": msim.PinnedBuffer(n, np.uint32)}
            state = {k: b.array for k, b in bufs.items()}
            for k in ("pos", "heading", "rng"):
                state[k][...] = st[k]
        else:
            state = {k: st[k].copy() for k in ("pos", "heading", "rng")}
            state["count"] = np.empty(n, np.uint32)
        state["speed"] = st["speed"]
        pos, head, rng, speed = st["pos"].copy(), st["heading"].copy(), st["rng"].copy(), st["speed"].copy()
        for t in range(8):
            if t == 4:  # host edits between ticks
                who = rs.choice(n, 5000, replace=False)
                roads = rs.integers(0, road_map.num_roads, who.size)
                for arr in (state["pos"], pos):
                    arr[who] = road_map.road_pos[roads, :2]
                for arr in (state["heading"], head):
                    arr[who] = roads.astype(np.uint32) | np.uint32(0x80000000)
            sim.tick_host(state, neighbours=True, out=state)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 0, 0.1, 1,
                     threads=8)
            _same_state(state, {"pos": pos, "heading": head, "rng": rng}, f"at tick {t + 1}")
            ocnt, _, _ = orc.neighbours(pos, 2.0, 8, threads=8, with_idx=False)
            assert np.array_equal(state["count"], ocnt), f"counts differ at tick {t + 1}"
        assert np.any(rng != st["rng"])  # road-end draws happened, so the RNG write-back was exercised
        for b in bufs.values():
            b.free()


@pytest.mark.parametrize("side,n,cap", [(48, 200_000, 16), (16, 100_000, 8)])
@pytest.mark.parametrize("rng", ["pcg32", "xorshift128"])
def test_skin_query_matches_oracle(msim, orc, side, n, cap, rng):
    """Consecutive neighbour host ticks: from the second on, the query reads the index
    of the previous state with every box widened by the tick's largest displacement,
    and the index of the new state is built after it.  Counts and lists equal the
    oracle's every tick.  A host edit that moves entities by 1.5 m keeps that path
    (boxes widened by up to 1.66 m); one that moves them by 3 m (more than the radius)
    takes the usual order for that tick.  (48, 200,000): tiles of about 11 m, boxes within 2 x 2 tiles; (16,
    100,000): tiles of 2 x reach, so widened boxes span three tiles, and about 15
    neighbours per entity, beyond the eight kept in registers.)"""
    road_map = msim.RoadMap.lattice(side, 5)
    rk = {"xorshift128": 0, "pcg32": 1}[rng]
    radius = 2.0
    rs = np.random.default_rng(side)
    with msim.Simulation(road_map, n, rng=rng, dt=0.1, radius=radius, cap=cap, index="incremental") as sim:
        sim.init_entities(6, placement="fraction", speed=(1.0, 1.6))
        st = sim.get_state()
        state = {k: st[k].copy() for k in ("pos", "heading", "rng", "speed")}
        sim.reset_kernel_stats()
        skin = 0
        for t in range(10):
            if t == 4:  # the host moves 3,000 entities by 1.5 m
                who = rs.choice(n, 3000, replace=False)
                state["pos"][who, 0] += np.float32(1.5)
            if t == 7:  # and 100 by 3 m
                who = rs.choice(n, 100, replace=False)
                state["pos"][who, 1] -= np.float32(3.0)
            pos, head, rng_s = state["pos"].copy(), state["heading"].copy(), state["rng"].copy()
            got = sim.tick_host(state, neighbours=True, with_idx=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng_s, state["speed"], rk,
                     0.1, 1, threads=8)
            _same_state(got, {"pos": pos, "heading": head, "rng": rng_s}, f"at host tick {t + 1}")
            ocnt, oidx, _ = orc.neighbours(pos, radius, cap, threads=8)
            assert np.array_equal(got["count"], ocnt), f"counts differ at host tick {t + 1}"
            assert np.array_equal(got["idx"], oidx), f"lists differ at host tick {t + 1}"
            hs = sim.host_tick_stats()
            if t >= 1 and t != 7:
                skin += 1
            assert hs["host_ticks"] == t + 1
            assert hs["skin_queries"] == skin, (t, hs)
            if t == 4:
                assert 1.3 < hs["last_displacement"] <= radius
            if t == 7:
                assert hs["last_displacement"] > radius
            state = {"pos": got["pos"].copy(), "heading": got["heading"].copy(), "rng": got["rng"].copy(),
                     "speed": state["speed"]}
        # the context's exports follow the last query (its index has moved on since)
        cnt, idx = sim.get_neighbours()
        assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx)
        assert sim.collision_pairs() == int(ocnt.sum()) // 2
        # regular ticks on the same context, then host ticks again
        pos, head, rng_s = state["pos"].copy(), state["heading"].copy(), state["rng"].copy()
        for t in range(3):
            sim.step(1, neighbours=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng_s, state["speed"], rk,
                     0.1, 1, threads=8)
            _same_state(sim.get_state(), {"pos": pos, "heading": head, "rng": rng_s}, f"at regular tick {t + 1}")
            ocnt, oidx, _ = orc.neighbours(pos, radius, cap, threads=8)
            cnt, idx = sim.get_neighbours()
            assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx), f"neighbours differ at regular tick {t + 1}"
        state = {"pos": pos.copy(), "heading": head.copy(), "rng": rng_s.copy(), "speed": state["speed"]}
        for t in range(3):
            got = sim.tick_host(state, neighbours=True, with_idx=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng_s, state["speed"], rk,
                     0.1, 1, threads=8)
            _same_state(got, {"pos": pos, "heading": head, "rng": rng_s}, f"at host tick {t + 11}")
            ocnt, oidx, _ = orc.neighbours(pos, radius, cap, threads=8)
            assert np.array_equal(got["count"], ocnt) and np.array_equal(got["idx"], oidx)
            state = {"pos": got["pos"].copy(), "heading": got["heading"].copy(), "rng": got["rng"].copy(),
                     "speed": state["speed"]}
        assert sim.host_tick_stats()["skin_queries"] == skin + 2  # the first after the regular ticks sorts


def test_bad_heading_on_the_skin_path(msim, orc):
    """A bad heading in a host tick that takes the skin path (its move checks the
    headings itself): MSIM_ERR_OOB naming the first bad entity, the context's state
    kept, and the host ticks after it match the oracle."""
    road_map = msim.RoadMap.lattice(24, 6)
    n = 150_000
    with msim.Simulation(road_map, n, rng="pcg32", dt=0.1, radius=2.0, cap=8, index="incremental") as sim:
        sim.init_entities(4, placement="fraction", speed=(1.0, 1.6))
        st = sim.get_state()
        state = {k: st[k].copy() for k in ("pos", "heading", "rng", "speed")}
        for _ in range(2):
            got = sim.tick_host(state, neighbours=True)
            state = {"pos": got["pos"].copy(), "heading": got["heading"].copy(), "rng": got["rng"].copy(),
                     "speed": state["speed"]}
        assert sim.host_tick_stats()["skin_queries"] == 1
        before = sim.get_state()
        bad = {k: v.copy() for k, v in state.items()}
        bad["heading"][[140_001, 70_123]] = road_map.num_roads + 5  # chunks 3 and 2
        with pytest.raises(msim.MsimError) as e:
            sim.tick_host(bad, neighbours=True)
        assert e.value.code == 2 and "70123" in str(e.value)
        after = sim.get_state()
        for k in before:
            assert np.array_equal(before[k], after[k])
        pos, head, rng = state["pos"].copy(), state["heading"].copy(), state["rng"].copy()
        for t in range(3):
            got = sim.tick_host(state, neighbours=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, state["speed"], 1,
                     0.1, 1, threads=8)
            _same_state(got, {"pos": pos, "heading": head, "rng": rng}, f"at host tick {t + 1} after the error")
            ocnt, _, _ = orc.neighbours(pos, 2.0, 8, threads=8, with_idx=False)
            assert np.array_equal(got["count"], ocnt), f"counts differ at host tick {t + 1} after the error"
            state = {"pos": got["pos"].copy(), "heading": got["heading"].copy(), "rng": got["rng"].copy(),
                     "speed": state["speed"]}
