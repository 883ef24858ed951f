"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Imported only by tests/, by __graft_entry__.smoke() and by bench.py's CPU
baseline / reference arm.  Wraps oracle/liboracle.so (the C restatement of
random_move.comp) and, when it was built here, oracle/_ref/libref_quadtree.so
(the reference's own CPU quad tree from shader_validation/src/main.cpp).
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_LIB = None
_REF = None

u32p = ctypes.POINTER(ctypes.c_uint32)
f32p = ctypes.POINTER(ctypes.c_float)


def _p(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype)) if a is not None else None


def lib():
    global _LIB
    if _LIB is None:
        path = HERE / "liboracle.so"
        if not path.exists():
            import importlib.util
            spec = importlib.util.spec_from_file_location("build_oracle", HERE / "build_oracle.py")
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build_oracle()
        L = ctypes.CDLL(str(path))
        L.oracle_xs128_next.argtypes = [u32p]
        L.oracle_xs128_next.restype = ctypes.c_uint32
        L.oracle_pcg32_next.argtypes = [u32p]
        L.oracle_pcg32_next.restype = ctypes.c_uint32
        L.oracle_pcg32_seed.argtypes = [u32p, ctypes.c_uint64, ctypes.c_uint64]
        L.oracle_next_float.argtypes = [ctypes.c_uint32]
        L.oracle_next_float.restype = ctypes.c_float
        L.oracle_ranged.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]
        L.oracle_ranged.restype = ctypes.c_uint32
        L.oracle_rng_seq.argtypes = [ctypes.c_uint32, u32p, ctypes.c_uint32, u32p]
        L.oracle_splitmix64.argtypes = [ctypes.c_uint64]
        L.oracle_splitmix64.restype = ctypes.c_uint64
        L.oracle_draw.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint64]
        L.oracle_draw.restype = ctypes.c_uint64
        L.oracle_init_entities.argtypes = [ctypes.c_uint32, f32p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                                           ctypes.c_uint32, ctypes.c_float, ctypes.c_float, f32p, u32p, u32p, f32p]
        L.oracle_step.argtypes = [ctypes.c_uint32, f32p, u32p, ctypes.c_uint32, u32p, ctypes.c_uint32,
                                  ctypes.c_uint32, ctypes.c_float, f32p, ctypes.c_uint32, f32p, u32p, u32p, f32p,
                                  ctypes.c_int]
        L.oracle_neighbours.argtypes = [ctypes.c_uint32, f32p, ctypes.c_float, ctypes.c_uint32, u32p, u32p,
                                        ctypes.c_int]
        L.oracle_neighbours.restype = ctypes.c_uint64
        L.oracle_in_range.argtypes = [ctypes.c_float] * 5
        L.oracle_in_range.restype = ctypes.c_int
        L.oracle_lattice_new.argtypes = [ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float, ctypes.c_float,
                                         ctypes.c_float]
        L.oracle_lattice_new.restype = ctypes.c_void_p
        L.oracle_lattice_info.argtypes = [ctypes.c_void_p, u32p, u32p, f32p, f32p]
        L.oracle_lattice_copy.argtypes = [ctypes.c_void_p, f32p, u32p, u32p]
        L.oracle_lattice_free.argtypes = [ctypes.c_void_p]
        _LIB = L
    return _LIB


def ref_lib():
    """The reference's own CPU quad tree, or None when it was not built here."""
    global _REF
    if _REF is None:
        path = HERE / "_ref" / "libref_quadtree.so"
        if not path.exists():
            return None
        try:
            R = ctypes.CDLL(str(path))
        except OSError:  # built on another architecture
            return None
        R.ref_max_entities.restype = ctypes.c_int
        R.ref_lower_sets.argtypes = [ctypes.c_uint, f32p, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_uint, u32p, u32p, u32p, ctypes.c_uint]
        R.ref_lower_sets.restype = ctypes.c_int
        R.ref_collision_test_1.restype = ctypes.c_int
        R.ref_export_tree.argtypes = [ctypes.c_uint, f32p, ctypes.c_float, ctypes.c_float, ctypes.c_uint, u32p, u32p]
        R.ref_export_tree.restype = ctypes.c_int
        _REF = R
    return _REF


# ---- numpy conveniences -------------------------------------------------------

class OracleMap:
    """A road map as plain arrays: road_pos (R,4) f32, road_conn (R,4) u32,
    connections (C,) u32, width, height (the fields the oracle's functions read)."""

    def __init__(self, road_pos, road_conn, connections, width, height):
        self.road_pos = road_pos
        self.road_conn = road_conn
        self.connections = connections
        self.width = float(width)
        self.height = float(height)

    @property
    def num_roads(self) -> int:
        return int(self.road_pos.shape[0])


def lattice(side: int, seed: int, spacing: float = 50.0, jitter: float = 10.0, keep_prob: float = 0.9) -> OracleMap:
    """The synthetic side x side lattice road map of the workloads (msim_oracle.c)."""
    L = lib()
    h = L.oracle_lattice_new(side, seed, spacing, jitter, keep_prob)
    if not h:
        raise ValueError("lattice arguments rejected (side 2..8192, 0 <= 2 jitter < spacing, keep_prob in (0, 1])")
    try:
        R, C = ctypes.c_uint32(), ctypes.c_uint32()
        w, hh = ctypes.c_float(), ctypes.c_float()
        L.oracle_lattice_info(h, ctypes.byref(R), ctypes.byref(C), ctypes.byref(w), ctypes.byref(hh))
        pos = np.empty((R.value, 4), np.float32)
        conn = np.empty((R.value, 4), np.uint32)
        cl = np.empty(C.value, np.uint32)
        L.oracle_lattice_copy(h, _p(pos, ctypes.c_float), _p(conn, ctypes.c_uint32), _p(cl, ctypes.c_uint32))
    finally:
        L.oracle_lattice_free(h)
    return OracleMap(pos, conn, cl, w.value, hh.value)


def rng_seq(kind: int, state, n: int):
    s = np.array(state, dtype=np.uint32).copy()
    out = np.zeros(n, dtype=np.uint32)
    lib().oracle_rng_seq(kind, _p(s, ctypes.c_uint32), n, _p(out, ctypes.c_uint32))
    return out, s


def pcg32_seed(initstate: int, initseq: int):
    s = np.zeros(4, dtype=np.uint32)
    lib().oracle_pcg32_seed(_p(s, ctypes.c_uint32), initstate, initseq)
    return s


def next_float(u: int) -> float:
    return lib().oracle_next_float(u)


def ranged(u: int, lo: int, hi: int) -> int:
    return lib().oracle_ranged(u, lo, hi)


def init_entities(road_pos, n, rng_kind, seed, placement, speed_min, speed_max):
    road_pos = np.ascontiguousarray(road_pos, dtype=np.float32)
    pos = np.zeros((n, 2), np.float32)
    head = np.zeros(n, np.uint32)
    rng = np.zeros((n, 4), np.uint32)
    speed = np.zeros(n, np.float32)
    lib().oracle_init_entities(road_pos.shape[0], _p(road_pos, ctypes.c_float), n, rng_kind, seed, placement,
                               speed_min, speed_max, _p(pos, ctypes.c_float), _p(head, ctypes.c_uint32),
                               _p(rng, ctypes.c_uint32), _p(speed, ctypes.c_float))
    return pos, head, rng, speed


def step(road_pos, road_conn, connections, pos, head, rng, speed, rng_kind, dt, ticks, factor=None, threads=None):
    """Runs `ticks` move ticks in place on (pos, head, rng)."""
    road_pos = np.ascontiguousarray(road_pos, dtype=np.float32)
    road_conn = np.ascontiguousarray(road_conn, dtype=np.uint32)
    connections = np.ascontiguousarray(connections, dtype=np.uint32)
    for a, dt_ in ((pos, np.float32), (head, np.uint32), (rng, np.uint32), (speed, np.float32)):
        assert a.dtype == dt_ and a.flags.c_contiguous
    if factor is not None:
        factor = np.ascontiguousarray(factor, dtype=np.float32)
    n = head.shape[0]
    lib().oracle_step(road_pos.shape[0], _p(road_pos, ctypes.c_float), _p(road_conn, ctypes.c_uint32),
                      connections.shape[0], _p(connections, ctypes.c_uint32), n, rng_kind, dt,
                      _p(factor, ctypes.c_float), ticks, _p(pos, ctypes.c_float), _p(head, ctypes.c_uint32),
                      _p(rng, ctypes.c_uint32), _p(speed, ctypes.c_float), threads or 1)


def neighbours(pos, radius, cap, threads=None, with_idx=True, out=None):
    """(count, idx, pairs) of the CPU-grid query; `out` = (count, idx) arrays to reuse."""
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    n = pos.shape[0]
    if out is not None:
        count, idx = out
        assert count.dtype == np.uint32 and count.shape == (n,) and count.flags.c_contiguous
        if not (with_idx and cap):
            idx = None
        else:
            assert idx.dtype == np.uint32 and idx.shape == (n, cap) and idx.flags.c_contiguous
    else:
        count = np.zeros(n, np.uint32)
        idx = np.zeros((n, cap), np.uint32) if (with_idx and cap) else None
    pairs = lib().oracle_neighbours(n, _p(pos, ctypes.c_float), radius, cap, _p(count, ctypes.c_uint32),
                                    _p(idx, ctypes.c_uint32), threads or 1)
    return count, idx, int(pairs)


def in_range(ax, ay, bx, by, r) -> bool:
    return bool(lib().oracle_in_range(ax, ay, bx, by, r))


def ref_lower_sets(pos, world_w, world_h, radius, node_cap=10, max_ids=256):
    """Per entity i: (distinct partners j < i, counter events, partner ids ascending)
    as found by the reference's own CPU quad tree."""
    R = ref_lib()
    if R is None:
        raise RuntimeError("reference quad tree not built (reference sources absent)")
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    n = pos.shape[0]
    lower = np.zeros(n, np.uint32)
    events = np.zeros(n, np.uint32)
    ids = np.full((n, max_ids), 0xFFFFFFFF, np.uint32)
    rc = R.ref_lower_sets(n, _p(pos, ctypes.c_float), world_w, world_h, radius, node_cap,
                          _p(lower, ctypes.c_uint32), _p(events, ctypes.c_uint32), _p(ids, ctypes.c_uint32), max_ids)
    if rc != 0:
        raise ValueError("too many entities for the reference's static arrays")
    return lower, events, ids


def density_adjoint(road_map, state, speed, factor, rng_kind, dt, ticks, grid, target, threads=None,
                    fp64_model=False, with_schedule=False):
    """FP64 loss, density and gradients (speed, factor) of the density calibration
    about the FP32 trajectory (or the FP64 model with the FP32 step's event
    schedule), see msim_oracle.h; with_schedule adds the event bits (n, ceil(ticks/32))."""
    L = lib()
    d = ctypes.POINTER(ctypes.c_double)
    L.oracle_density_adjoint.restype = ctypes.c_double
    L.oracle_density_adjoint.argtypes = [ctypes.c_uint32, f32p, u32p, ctypes.c_uint32, u32p, ctypes.c_uint32,
                                         ctypes.c_uint32, ctypes.c_float, ctypes.c_uint32, f32p, u32p, u32p, f32p,
                                         f32p, ctypes.c_float, ctypes.c_float, ctypes.c_uint32, ctypes.c_uint32, f32p,
                                         d, d, d, ctypes.c_int, u32p, ctypes.c_int]
    rp = np.ascontiguousarray(road_map.road_pos, np.float32)
    rc = np.ascontiguousarray(road_map.road_conn, np.uint32)
    cl = np.ascontiguousarray(road_map.connections, np.uint32)
    pos0 = np.ascontiguousarray(state["pos"], np.float32)
    head0 = np.ascontiguousarray(state["heading"], np.uint32)
    rng0 = np.ascontiguousarray(state["rng"], np.uint32)
    speed = np.ascontiguousarray(speed, np.float32)
    factor = np.ascontiguousarray(factor, np.float32)
    target = np.ascontiguousarray(target, np.float32)
    n = head0.shape[0]
    G = grid[0] * grid[1]
    dens = np.zeros(G, np.float64)
    gs = np.zeros(n, np.float64)
    gf = np.zeros(rp.shape[0], np.float64)
    sched = np.zeros((n, (ticks + 31) // 32), np.uint32) if with_schedule else None
    loss = L.oracle_density_adjoint(rp.shape[0], _p(rp, ctypes.c_float), _p(rc, ctypes.c_uint32), cl.shape[0],
                                    _p(cl, ctypes.c_uint32), n, rng_kind, dt, ticks, _p(pos0, ctypes.c_float),
                                    _p(head0, ctypes.c_uint32), _p(rng0, ctypes.c_uint32), _p(speed, ctypes.c_float),
                                    _p(factor, ctypes.c_float), road_map.width, road_map.height, grid[0], grid[1],
                                    _p(target, ctypes.c_float), _p(dens, ctypes.c_double), _p(gs, ctypes.c_double),
                                    _p(gf, ctypes.c_double), int(bool(fp64_model)), _p(sched, ctypes.c_uint32),
                                    threads or cpu_count())
    if with_schedule:
        return loss, dens, gs, gf, sched
    return loss, dens, gs, gf


def ref_export_tree(pos, world_w, world_h, node_cap=10):
    """The reference quad tree (max depth 8) after inserting pos in order: (nodes
    (21845, 16) uint32 words, links (n, 5) uint32 words)."""
    R = ref_lib()
    if R is None:
        raise RuntimeError("reference quad tree not built (reference sources absent)")
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    nodes = np.zeros((21845, 16), np.uint32)
    links = np.zeros((pos.shape[0], 5), np.uint32)
    rc = R.ref_export_tree(pos.shape[0], _p(pos, ctypes.c_float), world_w, world_h, node_cap,
                           _p(nodes, ctypes.c_uint32), _p(links, ctypes.c_uint32))
    if rc != 0:
        raise ValueError("too many entities for the reference's static arrays")
    return nodes, links


def cpu_count() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1
