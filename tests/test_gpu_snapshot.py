"""SoA state snapshot and resume (msim_save_state / msim_load_state): a run resumed
from a snapshot continues bit-exact with the run that wrote it, neighbour sets
included; snapshots of another configuration and damaged files are rejected."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_snapshot_resume_is_bit_exact(msim, tmp_path):
    rm = msim.RoadMap.lattice(40, 8)
    n = 50_000
    snap = tmp_path / "state.msim"
    with msim.Simulation(rm, n, rng="pcg32", dt=0.1, radius=2.0, cap=16) as a:
        a.init_entities(3, placement="fraction", speed=(1.0, 1.6))
        a.step(37, neighbours=True)
        a.save_state(snap)
        a.step(25, neighbours=True)
        ref = a.get_state()
        rcnt, ridx = a.get_neighbours()
        rpairs = a.collision_pairs()
    with msim.Simulation(rm, n, rng="pcg32", dt=0.1, radius=2.0, cap=16) as b:
        b.load_state(snap)
        assert b.tick == 37
        b.step(25, neighbours=True)
        st = b.get_state()
        cnt, idx = b.get_neighbours()
        assert b.tick == 62
        for k in ("pos", "heading", "rng", "speed"):
            assert np.array_equal(st[k].view(np.uint32), ref[k].view(np.uint32)), k
        assert np.array_equal(cnt, rcnt) and np.array_equal(idx, ridx) and b.collision_pairs() == rpairs


def test_snapshot_rejects_other_configurations(msim, tmp_path):
    rm = msim.RoadMap.lattice(16, 2)
    snap = tmp_path / "s.msim"
    with msim.Simulation(rm, 1000, rng="pcg32", dt=0.1, radius=2.0, cap=8) as a:
        a.init_entities(1)
        a.save_state(snap)
    with msim.Simulation(rm, 1001, rng="pcg32", dt=0.1, radius=2.0, cap=8) as b:
        with pytest.raises(msim.MsimError):
            b.load_state(snap)  # other entity count
    with msim.Simulation(rm, 1000, rng="xorshift128", dt=0.1, radius=2.0, cap=8) as b:
        with pytest.raises(msim.MsimError):
            b.load_state(snap)  # other RNG
    data = snap.read_bytes()
    (tmp_path / "short.msim").write_bytes(data[: len(data) // 2])
    (tmp_path / "junk.msim").write_bytes(b"not a snapshot" * 10)
    with msim.Simulation(rm, 1000, rng="pcg32", dt=0.1, radius=2.0, cap=8) as b:
        for bad in ("short.msim", "junk.msim", "missing.msim"):
            with pytest.raises(msim.MsimError):
                b.load_state(tmp_path / bad)
        b.load_state(snap)  # still usable
        b.step(2, neighbours=True)
        b.sync()
