"""Batched ensemble: one persistent launch over many instances, bit-identical to
running every instance alone with the single-context move path."""
import numpy as np
import pytest


def _instances(msim, count, seed, side_range=(16, 48), entity_range=(1_000, 20_000)):
    sides, ents, seeds = msim.ensemble_config(count, seed, side_range, entity_range)
    maps = [msim.RoadMap.lattice(s, sd) for s, sd in zip(sides, seeds)]
    return maps, ents, seeds


def test_ensemble_config_is_deterministic(msim):
    a = msim.ensemble_config(512, 20261203)
    b = msim.ensemble_config(512, 20261203)
    assert a == b
    sides, ents, seeds = a
    assert min(sides) >= 16 and max(sides) <= 256 and min(ents) >= 1000 and max(ents) < 200_000
    assert seeds[0] == 20261203 and seeds[-1] == 20261203 + 511
    assert 10e6 < sum(ents) < 35e6  # expectation ~19.2M


def _alone(msim, road_map, n, seed, ticks, rng):
    with msim.Simulation(road_map, n, rng=rng, dt=0.1, radius=2.0, cap=0) as sim:
        sim.init_entities(seed, placement="fraction", speed=(1.0, 1.6))
        sim.step(ticks)
        return sim.get_state()


@pytest.mark.gpu
@pytest.mark.parametrize("rng", ["pcg32", "xorshift128"])
def test_batch_matches_single_instances(msim, rng):
    maps, ents, seeds = _instances(msim, 20, 5)
    ticks = 300
    with msim.Batch(maps, ents, rng=rng, dt=0.1) as b:
        b.init_entities(seeds)
        b.step(ticks)  # graph-captured launch
        states = [b.get_state(i) for i in range(len(maps))]
        assert b.info()["launches"] == 1
    for i, (m, n, sd) in enumerate(zip(maps, ents, seeds)):
        ref = _alone(msim, m, n, sd, ticks, rng)
        for k in ("pos", "heading", "rng", "speed"):
            assert np.array_equal(states[i][k].view(np.uint32), ref[k].view(np.uint32)), (i, k)


@pytest.mark.gpu
def test_batch_schedules_and_tuner(msim, tmp_path):
    maps, ents, seeds = _instances(msim, 12, 9)
    ref = None
    schedules = [(256, [0, 4000, 10000], [1, 2, 4], [256, 1024, 4096]),
                 (128, [0], [4], [512]),
                 (512, [0, 5000], [2, 1], [100_000, 777])]
    for sch in schedules:
        with msim.Batch(maps, ents) as b:
            b.init_entities(seeds)
            b.set_schedule(*sch)
            b.step(120)
            b.step(80)
            st = [b.get_state(i) for i in range(len(maps))]
        if ref is None:
            ref = st
        for a, c in zip(st, ref):
            for k in a:
                assert np.array_equal(a[k], c[k])
    cache = tmp_path / "tune.txt"
    with msim.Batch(maps, ents) as b:
        b.init_entities(seeds)
        before = [b.get_state(i) for i in range(len(maps))]
        b.tune(50, cache)
        after = [b.get_state(i) for i in range(len(maps))]
        for x, y in zip(before, after):  # tuning leaves the state unchanged
            for k in x:
                assert np.array_equal(x[k], y[k])
        tuned = b.schedule()
        b.step(200)
        st = [b.get_state(i) for i in range(len(maps))]
    for a, c in zip(st, ref):
        for k in a:
            assert np.array_equal(a[k], c[k])
    assert cache.read_text().count("\n") == 1
    with msim.Batch(maps, ents) as b:  # a cache hit gives the same schedule
        b.init_entities(seeds)
        b.tune(50, cache)
        assert b.schedule() == tuned
    assert cache.read_text().count("\n") == 1
