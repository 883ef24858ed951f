"""Per-tick parity of the CUDA path (through the C ABI) against the CPU oracle.

Integer state (headings, RNG states, neighbour ids and counts) must be equal;
positions are compared bit for bit (the move step has no FMA contraction and
uses correctly rounded divide and square root, so the tolerance is 0 m).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POS_TOL_M = 0.0  # bit-exact


def _assert_state(st, pos, head, rng, what=""):
    assert np.array_equal(st["heading"], head), f"headings differ {what}"
    assert np.array_equal(st["rng"], rng), f"RNG states differ {what}"
    if POS_TOL_M == 0.0:
        bad = np.nonzero(st["pos"].view(np.uint32) != pos.view(np.uint32))[0]
        assert bad.size == 0, f"positions differ {what}: first at entity {bad[:5]} {st['pos'][bad[:3]]} vs {pos[bad[:3]]}"
    else:
        np.testing.assert_allclose(st["pos"], pos, atol=POS_TOL_M, rtol=0)


def _oracle_state(orc, road_map, n, rng_kind, seed, placement, speed):
    return orc.init_entities(road_map.road_pos, n, rng_kind, seed, placement, speed[0], speed[1])


@pytest.mark.parametrize("rng_name,rng_kind", [("xorshift128", 0), ("pcg32", 1)])
@pytest.mark.parametrize("placement,pl", [("start", 0), ("fraction", 1)])
def test_init_matches_oracle(msim, orc, rng_name, rng_kind, placement, pl):
    road_map = msim.RoadMap.lattice(24, 3)
    n = 5000
    with msim.Simulation(road_map, n, rng=rng_name, dt=0.1, radius=2.0) as sim:
        sim.init_entities(99, placement=placement, speed=(1.0, 1.6))
        st = sim.get_state()
    pos, head, rng, speed = _oracle_state(orc, road_map, n, rng_kind, 99, pl, (1.0, 1.6))
    _assert_state(st, pos, head, rng, "after init")
    assert np.array_equal(st["speed"].view(np.uint32), speed.view(np.uint32))


@pytest.mark.parametrize("rng_name,rng_kind", [("xorshift128", 0), ("pcg32", 1)])
def test_plain_config_1000_ticks(msim, orc, rng_name, rng_kind):
    """Plain config: 10,000 entities on the 32x32 lattice, 1,000 ticks at dt = 0.1."""
    road_map = msim.RoadMap.lattice(32, 20261203)
    n, ticks = 10_000, 1000
    with msim.Simulation(road_map, n, rng=rng_name, dt=0.1, radius=2.0, cap=64) as sim:
        sim.init_entities(20261203, placement="fraction", speed=(1.0, 1.6))
        pos, head, rng, speed = _oracle_state(orc, road_map, n, rng_kind, 20261203, 1, (1.0, 1.6))
        # first per tick, then in multi-tick launches
        for t in range(20):
            sim.step(1)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, rng_kind, 0.1, 1)
            _assert_state(sim.get_state(), pos, head, rng, f"at tick {t + 1}")
        sim.step(ticks - 20)
        orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, rng_kind, 0.1,
                 ticks - 20, threads=8)
        _assert_state(sim.get_state(), pos, head, rng, f"at tick {ticks}")
        assert sim.tick == ticks
    # the run must have exercised road-end events with random choices
    assert np.any(rng != _oracle_state(orc, road_map, n, rng_kind, 20261203, 1, (1.0, 1.6))[2])


@pytest.mark.parametrize("rng_name,rng_kind,resort,index",
                         [("pcg32", 1, 3, "incremental"), ("xorshift128", 0, 1, "incremental"),
                          ("pcg32", 1, 1000, "incremental"), ("pcg32", 1, 3, "full"), ("xorshift128", 0, 1000, "auto")])
def test_neighbour_ticks_every_tick(msim, orc, rng_name, rng_kind, resort, index):
    """Move + index + neighbour query, compared every tick (states, counts, id lists);
    the index updated from the previous order, or fully re-sorted every tick."""
    road_map = msim.RoadMap.lattice(20, 5)
    n, ticks, cap, radius = 12_345, 40, 64, 2.0
    with msim.Simulation(road_map, n, rng=rng_name, dt=0.1, radius=radius, cap=cap, resort_interval=resort,
                         index=index) as sim:
        sim.init_entities(7, placement="fraction", speed=(1.0, 1.6))
        pos, head, rng, speed = _oracle_state(orc, road_map, n, rng_kind, 7, 1, (1.0, 1.6))
        for t in range(ticks):
            sim.step(1, neighbours=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, rng_kind, 0.1, 1)
            _assert_state(sim.get_state(), pos, head, rng, f"at tick {t + 1}")
            cnt, idx = sim.get_neighbours()
            ocnt, oidx, opairs = orc.neighbours(pos, radius, cap, threads=8)
            assert np.array_equal(cnt, ocnt), f"neighbour counts differ at tick {t + 1}"
            assert np.array_equal(idx, oidx), f"neighbour lists differ at tick {t + 1}"
            assert sim.collision_pairs() == opairs
        assert cnt.sum() > 0


@pytest.mark.parametrize("cell,passes", [(2.05, 3), (6.0, 3), (400.0, 2)])
def test_sort_pass_counts(msim, orc, cell, passes):
    """Tile sizes that give 2 and 3 radix passes (12- to 24-bit keys: tile Morton
    code plus up to 6 y-band bits)."""
    road_map = msim.RoadMap.lattice(64, 13)
    n, ticks = 150_000, 12
    with msim.Simulation(road_map, n, rng="pcg32", dt=0.1, radius=2.0, cap=32, cell_size=cell,
                         resort_interval=5) as sim:
        assert sim.info()["sort_passes"] == passes
        sim.init_entities(21, placement="fraction", speed=(1.0, 1.6))
        pos, head, rng, speed = _oracle_state(orc, road_map, n, 1, 21, 1, (1.0, 1.6))
        for t in range(ticks):
            sim.step(1, neighbours=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 1, 0.1, 1,
                     threads=8)
            if t % 4 == 3:
                _assert_state(sim.get_state(), pos, head, rng, f"at tick {t + 1}")
                cnt, idx = sim.get_neighbours()
                ocnt, oidx, opairs = orc.neighbours(pos, 2.0, 32, threads=8)
                assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx)
                assert sim.collision_pairs() == opairs


def test_scale_config_full_size(msim, orc):
    """16,000,000 entities on the 1024x1024 lattice (3 radix passes): states bit-exact
    and neighbour counts equal to the oracle after 3 neighbour ticks; pair count =
    half the count sum (symmetry)."""
    road_map = msim.RoadMap.lattice(1024, 20261203)
    n, ticks = 16_000_000, 3
    with msim.Simulation(road_map, n, rng="pcg32", dt=0.1, radius=2.0, cap=64) as sim:
        assert sim.info()["sort_passes"] == 3
        sim.init_entities(20261203, placement="fraction", speed=(1.0, 1.6))
        sim.step(ticks, neighbours=True)
        st = sim.get_state()
        cnt, _ = sim.get_neighbours(with_idx=False)
        pairs = sim.collision_pairs()
    pos, head, rng, speed = _oracle_state(orc, road_map, n, 1, 20261203, 1, (1.0, 1.6))
    orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 1, 0.1, ticks,
             threads=16)
    _assert_state(st, pos, head, rng, f"at tick {ticks}")
    ocnt, _, opairs = orc.neighbours(pos, 2.0, 0, threads=16, with_idx=False)
    assert np.array_equal(cnt, ocnt)
    assert pairs == opairs and 2 * pairs == int(cnt.sum())


def test_reference_mode_test_map(msim, orc):
    """test_map.json semantics: SPEED 1.4 per tick, xorshift128, R = 10, including the
    draw that reads one past the connection list (pad entry)."""
    import json
    from pathlib import Path

    g = np.load(Path(__file__).parent / "golden" / "test_map.npz")
    road_map = msim.RoadMap(g["road_pos"], g["road_conn"], g["connections"], float(g["width"]), float(g["height"]))
    n, ticks = 2000, 300
    with msim.Simulation(road_map, n, rng="xorshift128", dt=1.0, radius=10.0, cap=16, resort_interval=4) as sim:
        sim.init_entities(1, placement="start", speed=(1.4, 1.4))
        pos, head, rng, speed = _oracle_state(orc, road_map, n, 0, 1, 0, (1.4, 1.4))
        for t in range(ticks):
            sim.step(1, neighbours=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 0, 1.0, 1)
            if t % 10 == 9:
                _assert_state(sim.get_state(), pos, head, rng, f"at tick {t + 1}")
                cnt, idx = sim.get_neighbours()
                ocnt, oidx, _ = orc.neighbours(pos, 10.0, 16, threads=8)
                assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx)
        # every road must have been used
        assert set(np.unique(head & 0x7FFFFFFF)) == {0, 1, 2, 3}


def test_plain_neighbours_config_sampled(msim, orc):
    """1,000,000 entities on the 256x256 lattice, R = 2.0, cap 64: state and
    neighbour sets after 10 ticks (the full 500-tick run is in bench.py)."""
    road_map = msim.RoadMap.lattice(256, 20261203)
    n, ticks = 1_000_000, 10
    with msim.Simulation(road_map, n, rng="pcg32", dt=0.1, radius=2.0, cap=64) as sim:
        sim.init_entities(20261203, placement="fraction", speed=(1.0, 1.6))
        pos, head, rng, speed = _oracle_state(orc, road_map, n, 1, 20261203, 1, (1.0, 1.6))
        sim.step(ticks, neighbours=True)
        orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 1, 0.1, ticks,
                 threads=16)
        _assert_state(sim.get_state(), pos, head, rng, f"at tick {ticks}")
        cnt, idx = sim.get_neighbours()
        ocnt, oidx, opairs = orc.neighbours(pos, 2.0, 64, threads=16)
        assert np.array_equal(cnt, ocnt)
        assert np.array_equal(idx, oidx)
        assert sim.collision_pairs() == opairs


def test_edge_cases(msim, orc):
    road_map = msim.RoadMap.lattice(8, 1)
    # zero entities
    with msim.Simulation(road_map, 0, radius=2.0) as sim:
        sim.init_entities(1)
        sim.step(3, neighbours=True)
        sim.step(3)
        assert sim.get_state()["pos"].shape == (0, 2)
    # one entity, and a ragged count
    for n in (1, 4097, 129):
        with msim.Simulation(road_map, n, rng="pcg32", dt=0.1, radius=2.0, cap=8) as sim:
            sim.init_entities(3, placement="fraction", speed=(1.0, 1.6))
            pos, head, rng, speed = _oracle_state(orc, road_map, n, 1, 3, 1, (1.0, 1.6))
            sim.step(5, neighbours=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 1, 0.1, 5)
            _assert_state(sim.get_state(), pos, head, rng, f"n={n}")
            cnt, idx = sim.get_neighbours()
            ocnt, oidx, _ = orc.neighbours(pos, 2.0, 8)
            assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx)


def test_crowd_beyond_cap_and_radius_boundary(msim, orc):
    """Every entity at one point (count n-1 > cap: the cap smallest ids, ascending) and
    pairs exactly at distance R (excluded: the predicate is dist < R)."""
    road_map = msim.RoadMap.lattice(8, 1)
    n, cap = 300, 64
    rp = road_map.road_pos
    # speed 0: positions stay put, so the query sees exactly the set positions
    pos = np.repeat(rp[:1, :2], n, axis=0).astype(np.float32)
    pos[200:] = rp[5, :2]
    pos[250:] = rp[5, :2] + np.float32([2.0, 0.0])  # |dx| == R, dy == 0 -> distance == R -> not in range
    head = np.full(n, 0x80000000, np.uint32)
    head[200:] = 5 | 0x80000000
    rng = np.ones((n, 4), np.uint32)
    speed = np.zeros(n, np.float32)
    with msim.Simulation(road_map, n, dt=0.1, radius=2.0, cap=cap) as sim:
        sim.set_entities(pos, head, rng, speed)
        sim.step(1, neighbours=True)
        st = sim.get_state()
        cnt, idx = sim.get_neighbours()
    ocnt, oidx, _ = orc.neighbours(st["pos"], 2.0, cap)
    assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx)
    assert cnt[0] == 199 and np.array_equal(idx[0], np.arange(1, 65))
    assert cnt[210] == 49  # not the entities at distance exactly R


def test_coarse_tiles_many_entities_per_key(msim, orc):
    """200 m tiles on a 380 m lattice: 2 x 2 tiles and 64 bands give 256 keys for 3000
    entities, so the key-start table comes from the per-key search kernel."""
    road_map = msim.RoadMap.lattice(8, 2)
    n = 3000
    with msim.Simulation(road_map, n, rng="pcg32", dt=0.1, radius=2.0, cap=16, cell_size=200.0) as sim:
        assert (1 << sim.info()["key_bits"]) * 8 < n
        sim.init_entities(9, placement="fraction", speed=(1.0, 1.6))
        pos, head, rng, speed = _oracle_state(orc, road_map, n, 1, 9, 1, (1.0, 1.6))
        for _ in range(3):
            sim.step(2, neighbours=True)
            orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 1, 0.1, 2)
            _assert_state(sim.get_state(), pos, head, rng)
            cnt, idx = sim.get_neighbours()
            ocnt, oidx, opairs = orc.neighbours(pos, 2.0, 16)
            assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx)
            assert sim.collision_pairs() == opairs


@pytest.mark.parametrize("radius", [2.0, 0.3, 1.7, 5.55])
def test_radius_predicate_ulp_boundary(msim, orc, radius):
    """Pairs whose distance lies within a few ulps of R at random angles: the
    square-root-free predicate of the query decides every pair like the oracle's
    sqrt(dx*dx + dy*dy) < R."""
    road_map = msim.RoadMap.lattice(64, 3)
    rs = np.random.default_rng(int(radius * 100))
    spacing = 8.0 * radius
    nx = int(road_map.width // spacing) - 1
    ny = int(road_map.height // spacing) - 1
    pairs = min(nx * ny, 4000)
    cells = rs.choice(nx * ny, pairs, replace=False)
    anchor = np.stack([(cells % nx + 1) * spacing, (cells // nx + 1) * spacing], 1) + rs.uniform(0, 1, (pairs, 2))
    anchor = anchor.astype(np.float32)
    theta = rs.uniform(0, 2 * np.pi, pairs)
    d = radius * (1.0 + rs.integers(-4, 5, pairs) * 2.0 ** -23)
    partner = (anchor + np.stack([d * np.cos(theta), d * np.sin(theta)], 1)).astype(np.float32)
    pos = np.concatenate([anchor, partner]).astype(np.float32)
    n = pos.shape[0]
    head = np.zeros(n, np.uint32)
    rng = np.ones((n, 4), np.uint32)
    speed = np.zeros(n, np.float32)
    with msim.Simulation(road_map, n, dt=0.1, radius=radius, cap=4) as sim:
        sim.set_entities(pos, head, rng, speed)
        sim.step(1, neighbours=True)
        st = sim.get_state()
        cnt, idx = sim.get_neighbours()
    assert np.array_equal(st["pos"].view(np.uint32), pos.view(np.uint32))
    ocnt, oidx, _ = orc.neighbours(pos, radius, 4)
    assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx)
    inside = ocnt[:pairs]
    assert 0 < inside.sum() < pairs  # both sides of the boundary are exercised


def test_reference_quadtree_golden(msim, golden_dir):
    """Neighbour lower-counts against the reference's own CPU quad tree
    (shader_validation), from fixtures generated with the reference code."""
    g = np.load(golden_dir / "ref_quadtree.npz")
    for k in range(int(g["cases"])):
        pos = g[f"pos{k}"]
        world = g[f"world{k}"]
        radius = float(g[f"radius{k}"])
        ref = g[f"lower{k}"]
        n = pos.shape[0]
        a, b = np.float32(0.25) * world, np.float32(0.75) * world
        road_map = msim.RoadMap(np.array([[a[0], a[1], b[0], b[1]]], np.float32), np.zeros((1, 4), np.uint32),
                                np.zeros(0, np.uint32), float(world[0]), float(world[1]))
        with msim.Simulation(road_map, n, dt=1.0, radius=radius, cap=256) as sim:
            sim.set_entities(pos, np.full(n, 0x80000000, np.uint32), np.ones((n, 4), np.uint32),
                             np.zeros(n, np.float32))
            sim.step(1, neighbours=True)
            assert np.array_equal(sim.get_state()["pos"], pos)
            cnt, idx = sim.get_neighbours()
        assert cnt.max() <= 256
        ids = g[f"ids{k}"]
        for i in range(n):
            mine = idx[i, : cnt[i]]
            mine = mine[mine < i]
            assert mine.size == ref[i], f"case {k} entity {i}: {mine.size} partners below, reference {ref[i]}"
            assert np.array_equal(mine, ids[i, : ref[i]]), f"case {k} entity {i}: partner ids differ"


def test_entities_aos_export(msim, orc):
    road_map = msim.RoadMap.lattice(12, 2)
    n = 1000
    with msim.Simulation(road_map, n, dt=1.0, radius=10.0, cap=8) as sim:
        sim.init_entities(5)
        ents = sim.export_entities()
        assert np.all(ents["color"] == np.float32([1, 0, 0, 1]))
        sim.step(3, neighbours=True)
        st = sim.get_state()
        cnt, _ = sim.get_neighbours()
        ents = sim.export_entities()
    assert ents.dtype.itemsize == 64
    assert np.array_equal(ents["pos"], st["pos"])
    assert np.array_equal(ents["randomState"], st["rng"])
    assert np.array_equal(ents["roadIndex"], st["heading"] & 0x7FFFFFFF)
    assert np.all(ents["initialized"] == 1)
    rp = road_map.road_pos[ents["roadIndex"]]
    to_end = (st["heading"] >> 31).astype(bool)
    target = np.where(to_end[:, None], rp[:, 2:], rp[:, :2])
    assert np.array_equal(ents["target"], target)
    blue = np.float32([0, 0, 1, 1])
    green = np.float32([0, 1, 0, 1])
    assert np.array_equal(ents["color"][cnt > 0], np.broadcast_to(blue, ((cnt > 0).sum(), 4)))
    assert np.array_equal(ents["color"][cnt == 0], np.broadcast_to(green, ((cnt == 0).sum(), 4)))
    d = target - st["pos"]
    ln = np.sqrt((d * d).sum(1))
    moving = ln > 0
    np.testing.assert_allclose(np.sqrt((ents["direction"][moving] ** 2).sum(1)), 1.4, rtol=1e-5)


def test_error_paths(msim):
    road_map = msim.RoadMap.lattice(8, 1)
    with msim.Simulation(road_map, 10) as sim:
        with pytest.raises(msim.MsimError) as e:
            sim.get_neighbours()
        assert e.value.code == 1
        bad = np.full(10, road_map.num_roads, np.uint32)
        with pytest.raises(msim.MsimError) as e:
            sim.set_entities(np.zeros((10, 2), np.float32), bad, np.ones((10, 4), np.uint32))
        assert e.value.code == 2
    broken = msim.RoadMap(road_map.road_pos, road_map.road_conn, road_map.connections.copy(), road_map.width,
                          road_map.height)
    broken.connections[0] = 10**6
    with pytest.raises(msim.MsimError) as e:
        msim.Simulation(broken, 10)
    assert e.value.code == 2


@pytest.mark.parametrize("reuse", [False, True])
def test_determinism_and_profiling(msim, reuse):
    road_map = msim.RoadMap.lattice(64, 9)
    outs = []
    for _ in range(2):
        with msim.Simulation(road_map, 50_000, rng="pcg32", dt=0.1, radius=2.0, cap=64, resort_interval=5,
                             reuse=reuse) as sim:
            sim.init_entities(4, placement="fraction", speed=(1.0, 1.6))
            sim.set_profiling(True)
            sim.step(12, neighbours=True)
            stats = sim.kernel_stats()
            outs.append((sim.get_state(), sim.get_neighbours()))
    assert stats["k_query"]["launches"] == 12
    if reuse:  # one update, on tick 1 (a bound of 0.161 m per tick against a 2 m reach:
        # ticks 2-12 reuse it, their moves placing the positions by the update's ranks);
        # the re-ordering waits for an update
        assert stats["k_step"]["launches"] == 1 and stats["k_move"]["launches"] == 11
        assert stats["k_mark"]["launches"] == 1 and "k_gather" not in stats
        assert "k_permute" not in stats
    else:
        assert stats["k_step"]["launches"] == 12 and "k_move" not in stats
        assert stats["k_permute"]["launches"] == 2
    (s0, (c0, i0)), (s1, (c1, i1)) = outs
    for k in s0:
        assert np.array_equal(s0[k], s1[k])
    assert np.array_equal(c0, c1) and np.array_equal(i0, i1)


def test_quad_tree_export_through_context(msim, golden_dir):
    g = np.load(golden_dir / "ref_tree.npz")
    pos = g["pos"]
    n = pos.shape[0]
    w, h = float(g["world"][0]), float(g["world"][1])
    road_map = msim.RoadMap(np.float32([[0.25 * w, 0.25 * h, 0.75 * w, 0.75 * h]]), np.zeros((1, 4), np.uint32),
                            np.zeros(0, np.uint32), w, h)
    with msim.Simulation(road_map, n, dt=1.0, radius=2.0, cap=8) as sim:
        sim.set_entities(pos, np.full(n, 0x80000000, np.uint32), np.ones((n, 4), np.uint32), np.zeros(n, np.float32))
        sim.step(2, neighbours=True)
        nodes, links, used = sim.export_quad_tree()
    assert np.array_equal(nodes.view(np.uint32).reshape(-1, 16), g["nodes"])
    assert np.array_equal(links.view(np.uint32).reshape(-1, 5), g["links"])
