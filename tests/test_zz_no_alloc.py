"""msim_query_neighbours_noalloc: neighbour sets without any device allocation.

The entry point exists for callers that cannot call cudaMalloc where they need
neighbour sets (inside stream capture, under a host that owns all device memory,
in a tick loop that must not block in the allocator).  This test calls it through
the C ABI with device buffers the test itself owns and checks two calls in a row
against the context path (msim_set_entities + msim_step(MSIM_STEP_NEIGHBOURS) +
msim_get_neighbours): counts and ids must be equal (integer results, tolerance 0).
The file is collected last so that a run stopping at the first failure has run
every other test first; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 262144


def _noalloc(msim):
    fn = msim.lib().msim_query_neighbours_noalloc
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_uint32,
                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    return fn


def _positions(seed, n, w, h):
    rs = np.random.default_rng(seed)
    pos = rs.uniform([0, 0], [w, h], (n, 2)).astype(np.float32)
    k = n // 4  # dense clusters (counts above the cap) and points exactly R apart
    centres = rs.uniform([10, 10], [w - 10, h - 10], (40, 2))
    pos[:k] = (centres[rs.integers(0, 40, k)] + rs.normal(0, 0.8, (k, 2))).astype(np.float32)
    pos[k: k + 50] = pos[k]
    pos[k + 50: k + 60] = pos[k] + np.float32([2.0, 0.0])
    return np.clip(pos, 0, [w - 1e-3, h - 1e-3]).astype(np.float32)


def _context_path(msim, pos, w, h, radius, cap):
    n = pos.shape[0]
    road_map = msim.RoadMap(np.float32([[0.25 * w, 0.25 * h, 0.75 * w, 0.75 * h]]), np.zeros((1, 4), np.uint32),
                            np.zeros(0, np.uint32), w, h)
    with msim.Simulation(road_map, n, dt=1.0, radius=radius, cap=cap) as sim:
        sim.set_entities(pos, np.full(n, 0x80000000, np.uint32), np.ones((n, 4), np.uint32), np.zeros(n, np.float32))
        sim.step(1, neighbours=True)
        assert np.array_equal(sim.get_state()["pos"], pos)
        return sim.get_neighbours()


def test_noalloc_matches_context_path_twice():
    torch = pytest.importorskip("torch")
    import importlib

    msim = importlib.import_module("movement-sim_gb300")
    fn = _noalloc(msim)
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row; the second is smaller, so stale scratch from the first must not leak
    for n, w, h, radius, cap, seed in [(200_000, 900.0, 700.0, 2.0, 64, 1), (70_001, 400.0, 650.0, 3.5, 16, 2)]:
        pos = _positions(seed, n, w, h)
        d_pos = torch.from_numpy(pos).cuda()
        d_count = torch.full((n,), 0xDEAD, dtype=torch.int32, device="cuda")
        d_idx = torch.full((n, cap), 0xDEAD, dtype=torch.int32, device="cuda")
        d_status = torch.full((1,), 7, dtype=torch.int32, device="cuda")
        rc = fn(d_pos.data_ptr(), n, w, h, radius, cap, d_count.data_ptr(), d_idx.data_ptr(), d_status.data_ptr(),
                stream)
        assert rc == 0, msim.lib().msim_last_error()
        torch.cuda.synchronize()
        assert int(d_status.item()) == 0
        count = d_count.cpu().numpy().view(np.uint32)
        idx = d_idx.cpu().numpy().view(np.uint32)
        ref_count, ref_idx = _context_path(msim, pos, w, h, radius, cap)
        assert np.array_equal(count, ref_count)
        assert np.array_equal(idx, ref_idx)
        assert count.max() > cap  # the crowd exercises the cap


def test_noalloc_rejects_oversize():
    import importlib

    msim = importlib.import_module("movement-sim_gb300")
    fn = _noalloc(msim)
    rc = fn(None, MAX_N + 1, 100.0, 100.0, 2.0, 8, None, None, None, None)
    assert rc == 1
    assert b"no-allocation limit" in msim.lib().msim_last_error()
