"""Parity of the timed path at the workload sizes, against the CPU oracle.

The path under test is the one the benchmark times: the incremental index update,
index reuse between updates (queries on the last index with widened boxes), the
query of tick t running on a second stream beside tick t+1's move and index update
(double-buffered index), and the re-ordering of the state at the first index update
after every 64 ticks.

* 1,000,000 entities on the 256 x 256 lattice, radius 2 m, cap 64, all 500 ticks:
  positions, headings, RNG states, neighbour counts and id lists compared after
  every tick (the reference runs its collision dispatch after every move dispatch,
  Simulator.cpp:227-235, random_move.comp:875-878).
* The same workload advanced in multi-tick calls (the query overlaps the next
  tick inside a call), compared at every call boundary, with the default
  re-ordering interval and with a re-ordering every 5 ticks.
* 16,000,000 entities on the 1024 x 1024 lattice for 135 ticks in multi-tick
  calls: two re-orderings run under the overlap; full state, counts and id lists
  compared after ticks 65, 129 and 135.

Integer state and id lists must be equal; positions bit for bit (tolerance 0 m).
This file sorts first among the GPU tests so that these runs happen even when a
later test stops the run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 20261203
DT = 0.1
SPEED = (1.0, 1.6)
RADIUS, CAP = 2.0, 64
THREADS = 16


def _compare(sim, orc, road_map, ost, buf, what):
    pos, head, rng, _ = ost
    st = sim.get_state(out=buf["state"])
    assert np.array_equal(st["heading"], head), f"headings differ {what}"
    assert np.array_equal(st["rng"], rng), f"RNG states differ {what}"
    bad = np.nonzero(np.any(st["pos"].view(np.uint32) != pos.view(np.uint32), axis=1))[0]
    assert bad.size == 0, f"positions differ {what}: {bad.size} entities, first {bad[:5]}"
    cnt, idx = sim.get_neighbours(out=(buf["cnt"], buf["idx"]))
    ocnt, oidx, opairs = orc.neighbours(pos, RADIUS, CAP, threads=THREADS, out=(buf["ocnt"], buf["oidx"]))
    if not np.array_equal(cnt, ocnt):
        bad = np.nonzero(cnt != ocnt)[0]
        raise AssertionError(f"neighbour counts differ {what}: {bad.size} entities, first {bad[:5]} "
                             f"{cnt[bad[:5]]} vs {ocnt[bad[:5]]}")
    n = idx.shape[0]
    step = 1 << 20  # row blocks: no full-size temporaries
    for a in range(0, n, step):
        if not np.array_equal(idx[a:a + step], oidx[a:a + step]):
            rows = a + np.nonzero(np.any(idx[a:a + step] != oidx[a:a + step], axis=1))[0]
            raise AssertionError(f"neighbour lists differ {what}: first rows {rows[:5]}")
    assert sim.collision_pairs() == opairs, f"pair counter differs {what}"
    return int(cnt.sum())


def _host_available_bytes():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except OSError:
        pass
    return None


def _buffers(n):
    return {"state": {"pos": np.empty((n, 2), np.float32), "heading": np.empty(n, np.uint32),
                      "rng": np.empty((n, 4), np.uint32)},
            "cnt": np.empty(n, np.uint32), "idx": np.empty((n, CAP), np.uint32),
            "ocnt": np.empty(n, np.uint32), "oidx": np.empty((n, CAP), np.uint32)}


def _setup(msim, orc, side, n, **kw):
    road_map = msim.RoadMap.lattice(side, SEED)
    sim = msim.Simulation(road_map, n, rng="pcg32", dt=DT, radius=RADIUS, cap=CAP, **kw)
    sim.init_entities(SEED, placement="fraction", speed=SPEED)
    ost = orc.init_entities(road_map.road_pos, n, 1, SEED, 1, SPEED[0], SPEED[1])
    return road_map, sim, ost


def _oracle_ticks(orc, road_map, ost, ticks):
    pos, head, rng, speed = ost
    orc.step(road_map.road_pos, road_map.road_conn, road_map.connections, pos, head, rng, speed, 1, DT, ticks,
             threads=THREADS)


def test_neighbours_config_every_tick_500(msim, orc):
    """1 M entities, 256 x 256 lattice: every one of the 500 ticks compared in full."""
    n, ticks = 1_000_000, 500
    road_map, sim, ost = _setup(msim, orc, 256, n)
    buf = _buffers(n)
    links = 0
    with sim:
        assert sim.info()["resort_interval"] == 64
        for t in range(ticks):
            sim.step(1, neighbours=True)
            _oracle_ticks(orc, road_map, ost, 1)
            links += _compare(sim, orc, road_map, ost, buf, f"at tick {t + 1}")
        assert sim.tick == ticks
    assert links > 0
    # road-end events with random choices happened
    assert np.any(ost[2] != orc.init_entities(road_map.road_pos, n, 1, SEED, 1, SPEED[0], SPEED[1])[2])


@pytest.mark.parametrize("resort", [0, 5])
def test_neighbours_config_multi_tick_calls(msim, orc, resort):
    """1 M entities for 500 ticks in calls of 2-12 ticks (query overlapping the next
    tick inside each call); compared at every call boundary.  resort 0 = the
    default interval (64), 5 = many re-orderings under the overlap."""
    n, ticks = 1_000_000, 500
    road_map, sim, ost = _setup(msim, orc, 256, n, resort_interval=resort)
    buf = _buffers(n)
    lengths = np.random.default_rng(resort + 1).integers(2, 13, ticks)
    done = 0
    with sim:
        for k in lengths:
            k = int(min(k, ticks - done))
            if k == 0:
                break
            sim.step(k, neighbours=True)
            _oracle_ticks(orc, road_map, ost, k)
            done += k
            _compare(sim, orc, road_map, ost, buf, f"at tick {done} (call of {k} ticks)")
        assert done == ticks and sim.tick == ticks


def test_scale_config_reorders_under_overlap(msim, orc):
    """16 M entities, 1024 x 1024 lattice: 135 ticks in three multi-tick calls;
    the two re-orderings (at the first index update after 64 ticks each) run inside
    the calls.  Full state, counts and id lists compared after ticks 65, 129 and
    135."""
    n = 16_000_000
    avail = _host_available_bytes()
    need = n * (2 * 4 * CAP + 64)  # two id-list arrays, states and counts
    if avail is not None and avail < 2 * need:
        pytest.skip(f"host memory: {avail >> 30} GiB available, the comparison needs about {need >> 30} GiB")
    road_map, sim, ost = _setup(msim, orc, 1024, n)
    buf = _buffers(n)
    with sim:
        info = sim.info()
        assert info["resort_interval"] == 64 and info["sort_passes"] == 3
        done = 0
        for k in (65, 64, 6):
            sim.step(k, neighbours=True)
            _oracle_ticks(orc, road_map, ost, k)
            done += k
            links = _compare(sim, orc, road_map, ost, buf, f"at tick {done}")
            assert links > 0
        assert sim.tick == 135


def test_batched_config_512_instances(msim, orc):
    """The batched ensemble: 512 instances (lattice side U{16..256}, entities
    log-U[1e3, 2e5], seed = index + 20261203), 1,000 ticks in one graph-captured
    persistent launch, with the tuner's schedule.  32 instances spread over every
    size class are compared bit for bit with running each alone (one context, the
    plain move path), and the largest of them also with the oracle."""
    sides, ents, seeds = msim.ensemble_config(512, SEED)
    maps = [msim.RoadMap.lattice(s, sd) for s, sd in zip(sides, seeds)]
    ticks = 1000
    order = np.argsort(ents)
    sample = sorted(set(int(order[k]) for k in np.linspace(0, len(order) - 1, 32).round().astype(int)))
    with msim.Batch(maps, ents, rng="pcg32", dt=DT) as b:
        b.init_entities(seeds, placement="fraction", speed=SPEED)
        b.tune(100)
        b.init_entities(seeds, placement="fraction", speed=SPEED)
        b.step(ticks)
        b.sync()
        states = {i: b.get_state(i) for i in sample}
    for i in sample:
        with msim.Simulation(maps[i], ents[i], rng="pcg32", dt=DT, radius=RADIUS, cap=0) as sim:
            sim.init_entities(seeds[i], placement="fraction", speed=SPEED)
            sim.step(ticks)
            ref = sim.get_state()
        for k in ("pos", "heading", "rng", "speed"):
            assert np.array_equal(states[i][k].view(np.uint32), ref[k].view(np.uint32)), (i, ents[i], k)
    big = max(sample, key=lambda i: ents[i])
    ost = orc.init_entities(maps[big].road_pos, ents[big], 1, seeds[big], 1, SPEED[0], SPEED[1])
    _oracle_ticks(orc, maps[big], ost, ticks)
    assert np.array_equal(states[big]["pos"].view(np.uint32), ost[0].view(np.uint32))
    assert np.array_equal(states[big]["heading"], ost[1]) and np.array_equal(states[big]["rng"], ost[2])


def test_adjoint_config_full_size(msim, orc):
    """Differentiable calibration at its workload size: 262,144 entities on the
    128 x 128 lattice, 2,000 ticks, 512 x 512 density grid, checkpoints every 100
    ticks, target density from hidden road factors U[0.7, 1.3].  Loss, density and
    both gradients against the FP64 CPU adjoint about the same FP32 trajectory:
    gradients within 1e-4 relative (norm-wise), loss within 1e-6, density within 1e-5."""
    torch = pytest.importorskip("torch")
    import importlib

    cal = importlib.import_module("movement-sim_gb300.calibration")
    rm = msim.RoadMap.lattice(128, SEED)
    n, T, grid = 262_144, 2000, (512, 512)
    calib = cal.Calibration(rm, n, T, dt=DT, rng="pcg32", checkpoint_interval=100, grid=grid, seed=SEED,
                            placement="fraction", speed=SPEED)
    with calib:
        hidden = np.random.default_rng(SEED).uniform(0.7, 1.3, rm.num_roads).astype(np.float32)
        target = torch.empty(grid[0] * grid[1], dtype=torch.float32, device="cuda")
        calib.forward(factor=torch.from_numpy(hidden).cuda(), density=target)
        st = calib.initial_state()
        speed = torch.from_numpy(st["speed"].copy()).cuda()
        factor = torch.ones(rm.num_roads, dtype=torch.float32, device="cuda")
        dens = torch.empty_like(target)
        loss = calib.forward(speed, factor, target, density=dens)
        gs = torch.empty(n, dtype=torch.float32, device="cuda")
        gf = torch.empty(rm.num_roads, dtype=torch.float32, device="cuda")
        calib.backward(gs, gf)
        gs64, gf64 = calib.gradients_f64()
    rl, rdens, rgs, rgf = orc.density_adjoint(rm, st, st["speed"], np.ones(rm.num_roads, np.float32), 1, DT, T, grid,
                                              target.cpu().numpy(), threads=THREADS)
    assert abs(loss - rl) <= 1e-6 * abs(rl)
    np.testing.assert_allclose(dens.cpu().numpy(), rdens, rtol=1e-5, atol=1e-7 * rdens.max())
    for g, r in ((gs64, rgs), (gf64, rgf)):
        err = np.linalg.norm(g - r) / np.linalg.norm(r)
        assert err < 1e-4, err
    np.testing.assert_array_equal(gs.cpu().numpy(), gs64.astype(np.float32))
    np.testing.assert_array_equal(gf.cpu().numpy(), gf64.astype(np.float32))


@pytest.mark.parametrize("n,side,ticks,with_idx", [(16_000_000, 1024, 4, False), (1_000_000, 256, 20, True)])
def test_host_tick_config_sizes(msim, orc, n, side, ticks, with_idx):
    """The end-to-end path the benchmark times: msim_tick_host in place (the same
    page-locked arrays for input and output; only positions and counts downloaded,
    the changed headings and RNG states written into the arrays by the move kernel).
    16 M entities: 4 host ticks, state and counts against the oracle after each; 1 M:
    20 host ticks, with the id lists too.  From the second host tick on, the query reads
    the previous state's index with widened boxes."""
    if n > 4_000_000:
        avail = _host_available_bytes()
        if avail is not None and avail < n * 200:
            pytest.skip(f"host memory: {avail >> 30} GiB available")
    road_map = msim.RoadMap.lattice(side, SEED)
    with msim.Simulation(road_map, n, rng="pcg32", dt=DT, radius=RADIUS, cap=CAP) as sim:
        sim.init_entities(SEED, placement="fraction", speed=SPEED)
        st = sim.get_state()
        bufs = {"pos": msim.PinnedBuffer((n, 2), np.float32), "heading": msim.PinnedBuffer(n, np.uint32),
                "rng": msim.PinnedBuffer((n, 4), np.uint32), "count": msim.PinnedBuffer(n, np.uint32)}
        if with_idx:
            bufs["idx"] = msim.PinnedBuffer((n, CAP), np.uint32)
        try:
            state = {k: b.array for k, b in bufs.items()}
            for k in ("pos", "heading", "rng"):
                state[k][...] = st[k]
            state["speed"] = st["speed"]
            ost = (st["pos"].copy(), st["heading"].copy(), st["rng"].copy(), st["speed"].copy())
            ocnt, oidx = np.empty(n, np.uint32), np.empty((n, CAP), np.uint32) if with_idx else None
            for t in range(ticks):
                sim.tick_host(state, neighbours=True, out=state)
                _oracle_ticks(orc, road_map, ost, 1)
                what = f"after host tick {t + 1}"
                assert np.array_equal(state["heading"], ost[1]), f"headings differ {what}"
                assert np.array_equal(state["rng"], ost[2]), f"RNG states differ {what}"
                assert np.array_equal(state["pos"].view(np.uint32), ost[0].view(np.uint32)), f"positions differ {what}"
                c, i, _ = orc.neighbours(ost[0], RADIUS, CAP if with_idx else 0, threads=THREADS, with_idx=with_idx,
                                         out=(ocnt, oidx))
                assert np.array_equal(state["count"], c), f"counts differ {what}"
                if with_idx:
                    assert np.array_equal(state["idx"], i), f"neighbour lists differ {what}"
            assert sim.tick == ticks
            # every host tick after the first queried the previous state's index (widened boxes)
            assert sim.host_tick_stats()["skin_queries"] == ticks - 1
        finally:
            for b in bufs.values():
                b.free()
