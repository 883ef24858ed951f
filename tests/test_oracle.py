"""CPU tests of the oracle: published known-answer sequences, hand-derived road
choices on test_map.json, and the neighbour predicate against the reference's own
CPU quad tree (shader_validation/src/main.cpp)."""
import subprocess
import sys

import numpy as np
import pytest

MARSAGLIA_XOR128 = [3701687786, 458299110, 2500872618, 3633119408, 516391518]
PCG32_DEMO_42_54 = [0xA15C02B7, 0x7B47F409, 0xBA1D3330, 0x83D2F293, 0xBFA4784B, 0xCBED606E]


def test_xorshift128_known_answer(orc):
    # Marsaglia, "Xorshift RNGs" (2003), xor128 with x,y,z,w = 123456789, 362436069,
    # 521288629, 88675123.  The shader's uvec4 keeps the newest word in .x and the
    # oldest in .w (random_move.comp:725-736), so state = (w, z, y, x).
    out, _ = orc.rng_seq(0, [88675123, 521288629, 362436069, 123456789], 5)
    assert list(out) == MARSAGLIA_XOR128


def test_pcg32_known_answer(orc):
    # pcg32 reference demo: pcg32_srandom_r(&rng, 42u, 54u), first six outputs
    out, _ = orc.rng_seq(1, orc.pcg32_seed(42, 54), 6)
    assert list(out) == PCG32_DEMO_42_54


def test_next_float_and_ranged_edges(orc):
    assert orc.next_float(0) == 0.0
    assert orc.next_float(0xFFFFFFFF) == 1.0  # float(2^32-1) rounds to 2^32
    assert orc.next_float(0x80000000) == 0.5
    # random_move.comp:743-746 with min=1, max=count returns 0..count
    assert orc.ranged(0, 1, 4) == 0
    assert orc.ranged(0xFFFFFFFF, 1, 4) == 4
    assert orc.ranged(0x80000000, 1, 3) == 2  # ceil(1 + 0.5*3) - 1
    f = np.float32
    for u in [1, 12345, 2**31 - 1, 2**31 + 7, 2**32 - 129, 2**32 - 128]:
        for cnt in [3, 4, 5, 7]:
            x = f(f(u) * f(2.0**-32))
            v = f(f(1.0) + f(x * f(cnt)))
            assert orc.ranged(u, 1, cnt) == int(np.ceil(v)) - 1


def _test_map(golden_dir):
    g = np.load(golden_dir / "test_map.npz")
    return g["road_pos"], g["road_conn"], g["connections"]


def test_test_map_road_choices_hand_derived(orc, golden_dir):
    """One entity per case on test_map.json, SPEED 1.4, reference mode."""
    rp, rc, cl = _test_map(golden_dir)
    f = np.float32
    # road 0 (5,5)->(50,50); arriving at (50,50): end list at 1 (count 4)
    u_state = np.array([88675123, 521288629, 362436069, 123456789], np.uint32)
    first = MARSAGLIA_XOR128[0]
    off = orc.ranged(first, 1, 4)
    assert off == int(np.ceil(f(1) + f(f(f(first) * f(2.0**-32)) * f(4)))) - 1
    expected_road = int(cl[1 + off])
    # new target: the end of the new road that is not (50,50) -> its start
    exp_head = expected_road if tuple(rp[expected_road, :2]) != (50.0, 50.0) else expected_road | 0x80000000
    pos = np.array([[49.5, 49.5]], np.float32)
    head = np.array([0 | 0x80000000], np.uint32)
    rng = u_state.reshape(1, 4).copy()
    speed = np.array([1.4], np.float32)
    orc.step(rp, rc, cl, pos, head, rng, speed, 0, 1.0, 1)
    assert tuple(pos[0]) == (50.0, 50.0)  # snapped: distance 0.707 <= 1.4
    assert head[0] == exp_head
    assert list(rng[0]) != list(u_state)  # one draw consumed
    # U-turn at road 0's start (count 1): no draw, heads for the end again
    pos = np.array([[5.5, 5.5]], np.float32)
    head = np.array([0], np.uint32)
    rng = u_state.reshape(1, 4).copy()
    orc.step(rp, rc, cl, pos, head, rng, speed, 0, 1.0, 1)
    assert tuple(pos[0]) == (5.0, 5.0) and head[0] == 0x80000000 and np.array_equal(rng[0], u_state)
    # far from the target: one step of exactly (d / |d|) * 1.4 in binary32
    pos = np.array([[5.0, 5.0]], np.float32)
    head = np.array([0x80000000], np.uint32)
    orc.step(rp, rc, cl, pos, head, rng, speed, 0, 1.0, 1)
    d = f(45.0)
    ln = f(np.sqrt(f(d * d) + f(d * d)))
    assert pos[0, 0] == f(f(5.0) + f(f(d / ln) * f(1.4)))


def test_test_map_pad_entry(orc, golden_dir):
    """Road 3's end list starts at 16 with count 4: a draw of 4 reads index 20, one past
    the 20-entry list; the pad entry repeats the last connection (road 0)."""
    rp, rc, cl = _test_map(golden_dir)
    assert len(cl) == 20 and rc[3, 2] == 16 and rc[3, 3] == 4
    # find a state whose first draw gives offset 4 (a quarter of full-width states do)
    rs = np.random.default_rng(1)
    for _ in range(1000):
        s = rs.integers(1, 2**32, 4, dtype=np.uint64).astype(np.uint32)
        u, _ = orc.rng_seq(0, s, 1)
        if orc.ranged(int(u[0]), 1, 4) == 4:
            break
    else:
        pytest.fail("no state with a draw of 4 found")
    pos = np.array([[50.5, 50.5]], np.float32)
    head = np.array([3 | 0x80000000], np.uint32)
    rng = s.reshape(1, 4).copy()
    orc.step(rp, rc, cl, pos, head, rng, np.array([1.4], np.float32), 0, 1.0, 1)
    assert head[0] & 0x7FFFFFFF == cl[19] == 0
    assert head[0] == 0  # road 0's end is (50,50), so the target is its start


def test_step_threads_agree(orc):
    import importlib

    msim = importlib.import_module("movement-sim_gb300")
    m = msim.RoadMap.lattice(16, 4)
    a = orc.init_entities(m.road_pos, 20_000, 1, 5, 1, 1.0, 1.6)
    b = [x.copy() for x in a]
    orc.step(m.road_pos, m.road_conn, m.connections, *a, 1, 0.1, 300, threads=1)
    orc.step(m.road_pos, m.road_conn, m.connections, *b, 1, 0.1, 300, threads=7)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_neighbours_bruteforce(orc):
    rs = np.random.default_rng(3)
    pos = rs.uniform(0, 60, (1500, 2)).astype(np.float32)
    pos[:40] = pos[0]  # a crowd at one point
    cnt, idx, pairs = orc.neighbours(pos, 2.5, 16, threads=3)
    d = np.sqrt(((pos[:, None, :].astype(np.float64) - pos[None]) ** 2).sum(-1))
    for i in range(0, 1500, 7):
        js = np.nonzero(d[i] < 2.5)[0]
        js = js[js != i]
        assert cnt[i] == js.size
        exp = np.full(16, 0xFFFFFFFF, np.uint32)
        exp[: min(16, js.size)] = js[:16]
        assert np.array_equal(idx[i], exp)
    assert pairs * 2 == cnt.sum()


def test_predicate_boundaries(orc):
    assert not orc.in_range(0.0, 0.0, 2.0, 0.0, 2.0)  # distance == R is out
    assert orc.in_range(0.0, 0.0, 1.9999999, 0.0, 2.0)
    assert orc.in_range(5.0, 5.0, 5.0, 5.0, 2.0)  # same point
    assert not orc.in_range(0.0, 0.0, 1.5, 1.5, 2.0)  # |dx|,|dy| <= R but distance > R


def test_reference_known_answer_test_runs():
    """run_collision_detection_test_1 of the reference (its asserts abort on failure)."""
    from oracle import oracle as o

    if o.ref_lib() is None:
        pytest.skip("reference sources absent: oracle/_ref not built")
    code = ("import sys; sys.path.insert(0, %r); from oracle import oracle as o; "
            "o.ref_lib().ref_collision_test_1(); print('ok')") % str(o.HERE.parent)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "run_collision_detection_test_1 was successful." in r.stdout


def test_oracle_matches_reference_quadtree_golden(orc, golden_dir):
    """Distinct neighbour sets (j < i) from the reference's CPU quad tree, stored as
    fixtures, against the oracle; and freshly from oracle/_ref when it is built."""
    g = np.load(golden_dir / "ref_quadtree.npz")
    for k in range(int(g["cases"])):
        pos, radius = g[f"pos{k}"], float(g[f"radius{k}"])
        lower, ids = g[f"lower{k}"], g[f"ids{k}"]
        cnt, idx, _ = orc.neighbours(pos, radius, 1024)
        for i in range(pos.shape[0]):
            mine = idx[i, : cnt[i]]
            mine = mine[mine < i]
            assert np.array_equal(mine, ids[i, : lower[i]]), (k, i)
        # the reference's collision counter counts repeated visits: never fewer than pairs
        assert np.all(g[f"events{k}"] >= lower)
    if orc.ref_lib() is not None:
        rs = np.random.default_rng(11)
        pos = rs.uniform(0, 120, (700, 2)).astype(np.float32)
        lower, events, ids = orc.ref_lower_sets(pos, 120.0, 120.0, 6.0)
        cnt, idx, _ = orc.neighbours(pos, 6.0, 1024)
        for i in range(700):
            mine = idx[i, : cnt[i]]
            assert np.array_equal(mine[mine < i], ids[i, : lower[i]])


def _calibration_case(orc, msim, n=1500, ticks=200, side=16, grid=(64, 64), seed=5):
    road_map = msim.RoadMap.lattice(side, seed)
    pos, head, rng, speed = orc.init_entities(road_map.road_pos, n, 1, seed, 1, 1.0, 1.6)
    state = {"pos": pos, "heading": head, "rng": rng}
    hidden = np.random.default_rng(seed).uniform(0.7, 1.3, road_map.num_roads).astype(np.float32)
    G = grid[0] * grid[1]
    _, target, _, _ = orc.density_adjoint(road_map, state, speed, hidden, 1, 0.1, ticks, grid,
                                          np.zeros(G, np.float32))
    return road_map, state, speed, target.astype(np.float32)


def test_fp64_adjoint_central_differences(orc, msim):
    """The FP64 adjoint against central differences (step 1e-3) of the smooth FP64
    model on 64 random parameters (32 speeds, 32 road factors) whose +-1e-3 runs
    keep the event schedule (no road-end event crossed)."""
    ticks, grid, h = 200, (64, 64), 1e-3
    road_map, state, speed, target = _calibration_case(orc, msim, ticks=ticks, grid=grid)
    factor = np.ones(road_map.num_roads, np.float32)

    def run(sp, fa):
        return orc.density_adjoint(road_map, state, sp, fa, 1, 0.1, ticks, grid, target, fp64_model=True,
                                   with_schedule=True)

    loss, _, gs, gf, sched = run(speed, factor)
    rs = np.random.default_rng(11)
    for kind, vec, grad in (("speed", speed, gs), ("factor", factor, gf)):
        checked = tried = 0
        rel = []
        for i in rs.permutation(vec.size):
            if checked == 32 or tried == 400:
                break
            tried += 1
            res, used = [], []
            for d in (h, -h):
                v = vec.copy()
                v[i] = np.float32(vec[i] + d)
                used.append(float(v[i]))
                out = run(v, factor) if kind == "speed" else run(speed, v)
                if not np.array_equal(out[4], sched):
                    break
                res.append(out[0])
            if len(res) < 2:
                continue
            fd = (res[0] - res[1]) / (used[0] - used[1])
            # the splat is piecewise bilinear: a +-1e-3 run whose positions cross a
            # cell-centre line sees the kink, hence the absolute term
            err = abs(fd - grad[i])
            assert err <= 2e-2 * abs(grad[i]) + 2e-3 * np.abs(grad).max(), (kind, i, fd, grad[i])
            rel.append(err / max(abs(grad[i]), 1e-300))
            checked += 1
        assert checked == 32, (kind, checked, tried)
        assert np.median(rel) < 1e-3, (kind, np.median(rel))
