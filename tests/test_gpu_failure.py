"""Failure detection, exercised without faulting the GPU (include/msim_debug.h).

* A bounded device wait that runs out: the look-back chain of the next index update
  is started at tile 1, so tile 1 waits for a tile 0 that never publishes.  With a
  short wait limit the kernel gives up, later index kernels skip their work,
  msim_sync reports MSIM_ERR_TIMEOUT, the entity state is intact, and the next
  neighbour tick rebuilds the index and matches the oracle again.
* A kernel launch that reports an error (injected on the host instead of the launch):
  msim_step returns MSIM_ERR_CUDA, the device is unharmed (msim_sync succeeds), and a
  caller that sets its state again continues bit-exact with the oracle.
* Device allocations that fail at every point of context creation: MSIM_ERR_NOMEM,
  nothing leaked, and creation succeeds once the injection is off.

The reference has no failure detection (its README asks users to turn off the GPU
hang check), so these have no reference counterpart.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SEED = 11
SPEED = (1.0, 1.6)


def _oracle(orc, rm, n):
    return orc.init_entities(rm.road_pos, n, 1, SEED, 1, SPEED[0], SPEED[1])


def _advance(orc, rm, ost, ticks):
    pos, head, rng, speed = ost
    orc.step(rm.road_pos, rm.road_conn, rm.connections, pos, head, rng, speed, 1, 0.1, ticks, threads=8)


def _same_state(sim, ost, what):
    st = sim.get_state()
    assert np.array_equal(st["heading"], ost[1]), f"headings differ {what}"
    assert np.array_equal(st["rng"], ost[2]), f"RNG states differ {what}"
    assert np.array_equal(st["pos"].view(np.uint32), ost[0].view(np.uint32)), f"positions differ {what}"


def _same_neighbours(sim, orc, ost, cap, what):
    cnt, idx = sim.get_neighbours()
    ocnt, oidx, opairs = orc.neighbours(ost[0], 2.0, cap, threads=8)
    assert np.array_equal(cnt, ocnt) and np.array_equal(idx, oidx), f"neighbours differ {what}"
    assert sim.collision_pairs() == opairs


@pytest.mark.parametrize("index", ["full", "auto"])
def test_wait_timeout_reports_and_recovers(msim, orc, index):
    """full: the first radix pass of a full sort; auto: the split of an incremental
    update (both chains have 8 tiles at 30,000 entities).  Index reuse off, so every
    neighbour tick updates the index (the next test covers it on)."""
    rm = msim.RoadMap.lattice(32, 3)
    n, cap = 30_000, 16
    ost = _oracle(orc, rm, n)
    with msim.Simulation(rm, n, rng="pcg32", dt=0.1, radius=2.0, cap=cap, index=index, resort_interval=4,
                         reuse=False) as sim:
        sim.init_entities(SEED, placement="fraction", speed=SPEED)
        sim.step(2, neighbours=True)
        _advance(orc, rm, ost, 2)
        _same_neighbours(sim, orc, ost, cap, "before the fault")
        sim.set_wait_limit(2048)
        sim.inject_fault(msim._capi.FAULT_SORT_TILE)
        sim.step(1, neighbours=True)
        with pytest.raises(msim.MsimError) as ei:
            sim.sync()
        assert ei.value.code == 4, str(ei.value)  # MSIM_ERR_TIMEOUT
        _advance(orc, rm, ost, 1)
        _same_state(sim, ost, "after the timed-out tick")  # the move ran, the state is intact
        sim.set_wait_limit(0)
        for t in range(6):  # full sort, then re-ordering and incremental updates again
            sim.step(1, neighbours=True)
            _advance(orc, rm, ost, 1)
            _same_state(sim, ost, f"{t + 1} ticks after recovery")
            _same_neighbours(sim, orc, ost, cap, f"{t + 1} ticks after recovery")
        sim.sync()


def test_wait_timeout_with_index_reuse(msim, orc):
    """With index reuse the armed fault waits for the next index update (ticks that
    reuse the index run none); that tick's wait gives up, msim_sync reports it, the
    state is intact, and the ticks after match the oracle again."""
    rm = msim.RoadMap.lattice(32, 3)
    n, cap = 30_000, 16
    ost = _oracle(orc, rm, n)
    with msim.Simulation(rm, n, rng="pcg32", dt=0.1, radius=2.0, cap=cap, resort_interval=4) as sim:
        sim.init_entities(SEED, placement="fraction", speed=SPEED)
        sim.step(3, neighbours=True)
        _advance(orc, rm, ost, 3)
        _same_neighbours(sim, orc, ost, cap, "before the fault")
        updates = sim.sort_stats()["index_updates"]
        sim.set_wait_limit(2048)
        sim.inject_fault(msim._capi.FAULT_SORT_TILE)
        for t in range(24):  # until the tick that updates the index
            sim.step(1, neighbours=True)
            _advance(orc, rm, ost, 1)
            if sim.sort_stats()["index_updates"] > updates:
                break
            _same_state(sim, ost, f"{t + 1} ticks after arming")
            _same_neighbours(sim, orc, ost, cap, f"{t + 1} ticks after arming (index reused)")
        else:
            raise AssertionError("no index update within 24 ticks")
        assert t >= 1  # at least one tick reused the index before
        with pytest.raises(msim.MsimError) as ei:
            sim.sync()
        assert ei.value.code == 4, str(ei.value)  # MSIM_ERR_TIMEOUT
        _same_state(sim, ost, "after the timed-out tick")
        sim.set_wait_limit(0)
        for t in range(8):
            sim.step(1, neighbours=True)
            _advance(orc, rm, ost, 1)
            _same_state(sim, ost, f"{t + 1} ticks after recovery")
            _same_neighbours(sim, orc, ost, cap, f"{t + 1} ticks after recovery")
        sim.sync()


@pytest.mark.parametrize("reuse,arg", [(False, 0), (False, 1), (False, 2), (False, 4), (False, 7),
                                       (True, 0), (True, 1), (True, 2), (True, 3)])
def test_injected_launch_failure(msim, orc, reuse, arg):
    """The (arg+1)-th launch of a 2-tick neighbour step fails on the host; the caller
    restores its state with msim_set_entities and continues bit-exact.  Without index
    reuse both ticks update the index; with it both reuse it (the move, placing the
    positions by the ranks of the last update, then the query)."""
    rm = msim.RoadMap.lattice(32, 4)
    n, cap = 20_000, 16
    ost = _oracle(orc, rm, n)
    with msim.Simulation(rm, n, rng="pcg32", dt=0.1, radius=2.0, cap=cap, reuse=reuse) as sim:
        sim.init_entities(SEED, placement="fraction", speed=SPEED)
        sim.step(1, neighbours=True)
        _advance(orc, rm, ost, 1)
        sim.inject_fault(msim._capi.FAULT_LAUNCH, arg)
        with pytest.raises(msim.MsimError) as ei:
            sim.step(2, neighbours=True)
        assert ei.value.code == 3, str(ei.value)  # MSIM_ERR_CUDA
        sim.sync()  # nothing happened on the device
        sim.set_entities(ost[0], ost[1], ost[2], ost[3])
        for t in range(4):
            sim.step(1, neighbours=True)
            _advance(orc, rm, ost, 1)
            _same_state(sim, ost, f"{t + 1} ticks after the failed launch")
            _same_neighbours(sim, orc, ost, cap, f"{t + 1} ticks after the failed launch")
        # a move-only step whose launch fails leaves the state as it was
        sim.inject_fault(msim._capi.FAULT_LAUNCH, 0)
        with pytest.raises(msim.MsimError):
            sim.step(5)
        sim.step(5)
        _advance(orc, rm, ost, 5)
        _same_state(sim, ost, "after a failed move-only launch")


def test_device_allocation_failure_everywhere(msim):
    """Creation fails cleanly at each of its device allocations and leaks nothing."""
    torch = pytest.importorskip("torch")
    L = msim.lib()
    rm = msim.RoadMap.lattice(16, 1)
    msim.Simulation(rm, 5000, radius=2.0, cap=8).close()  # the CUDA context exists from here on
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    failures = 0
    try:
        for after in range(0, 400):
            L.msim_debug_fail_device_alloc(after)
            try:
                sim = msim.Simulation(rm, 5000, radius=2.0, cap=8)
            except msim.MsimError as e:
                assert e.code == 5, str(e)  # MSIM_ERR_NOMEM
                failures += 1
                continue
            sim.close()
            break
        else:
            raise AssertionError("creation never succeeded")
        # the batch and the calibration context too
        for after in (0, 3, 9):
            L.msim_debug_fail_device_alloc(after)
            with pytest.raises(msim.MsimError) as ei:
                msim.Batch([rm, rm], [1000, 2000])
            assert ei.value.code == 5
    finally:
        L.msim_debug_fail_device_alloc(-1)
    assert failures >= 20  # every allocation point of msim_create was hit
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert abs(free0 - free1) < (16 << 20), f"device memory changed by {free0 - free1} bytes"
    with msim.Simulation(rm, 5000, rng="pcg32", dt=0.1, radius=2.0, cap=8) as sim:
        sim.init_entities(SEED, placement="fraction", speed=SPEED)
        sim.step(3, neighbours=True)
        sim.sync()


def test_set_device_checks_its_argument(msim):
    """msim_set_device selects the library's GPU (its own CUDA runtime does not follow
    the application's); ids outside the device count are rejected."""
    torch = pytest.importorskip("torch")
    count = torch.cuda.device_count()
    msim.set_device(0)
    for bad in (-1, count, count + 7):
        with pytest.raises(msim.MsimError) as ei:
            msim.set_device(bad)
        assert ei.value.code == 1  # MSIM_ERR_INVALID
    msim.set_device(0)
    rm = msim.RoadMap.lattice(16, 3)
    with msim.Simulation(rm, 2000, rng="pcg32", dt=0.1, radius=2.0, cap=8) as sim:
        sim.init_entities(1, placement="fraction", speed=SPEED)
        sim.step(2, neighbours=True)
        sim.sync()


def test_host_tick_background_update_timeout(msim, orc):
    """With consecutive neighbour host ticks the index of the new state is built after
    the tick's query, off the caller's path; a wait of that update that gives up is
    reported by the next call (MSIM_ERR_TIMEOUT, its moved state intact), and the host
    ticks after it match the oracle again (the index is rebuilt by a full sort)."""
    rm = msim.RoadMap.lattice(32, 3)
    n, cap = 150_000, 16
    ost = list(_oracle(orc, rm, n))
    with msim.Simulation(rm, n, rng="pcg32", dt=0.1, radius=2.0, cap=cap, index="incremental") as sim:
        sim.init_entities(SEED, placement="fraction", speed=SPEED)
        state = {k: v.copy() for k, v in sim.get_state().items()}

        def host_tick(what):
            nonlocal state
            got = sim.tick_host(state, neighbours=True, with_idx=True)
            _advance(orc, rm, ost, 1)
            assert np.array_equal(got["pos"].view(np.uint32), ost[0].view(np.uint32)), f"positions differ {what}"
            ocnt, oidx, _ = orc.neighbours(ost[0], 2.0, cap, threads=8)
            assert np.array_equal(got["count"], ocnt) and np.array_equal(got["idx"], oidx), f"neighbours differ {what}"
            state = {"pos": got["pos"].copy(), "heading": got["heading"].copy(), "rng": got["rng"].copy(),
                     "speed": state["speed"]}

        host_tick("at the first host tick")
        host_tick("at the second host tick")
        assert sim.host_tick_stats()["skin_queries"] == 1
        sim.set_wait_limit(2048)
        sim.inject_fault(msim._capi.FAULT_SORT_TILE)  # hits the index update after this tick's query
        host_tick("at the tick whose index update gives up")
        with pytest.raises(msim.MsimError) as ei:
            sim.tick_host(state, neighbours=True)
        assert ei.value.code == 4, str(ei.value)  # MSIM_ERR_TIMEOUT
        _advance(orc, rm, ost, 1)
        _same_state(sim, ost, "after the call that reported the timeout")
        sim.set_wait_limit(0)
        state = {k: v.copy() for k, v in sim.get_state().items()}
        for t in range(4):
            host_tick(f"{t + 1} host ticks after recovery")
        sim.sync()
