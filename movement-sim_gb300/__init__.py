"""GB300-native per-tick path of movement-sim: Python bindings over the C ABI.

Import with ``importlib.import_module("movement-sim_gb300")`` (the directory name
carries a hyphen).  Everything here calls libmsim.so through include/msim.h;
there is no CPU fallback.

* :class:`RoadMap` - a road graph in the reference map layout (Map.hpp:12-48):
  the JSON loader of Map.cpp:28-150, the writer of map/generate_map.py:152-160
  and the synthetic lattice generator.
* :class:`Simulation` - one device context (Simulator.cpp:44-106 init, sim_tick
  213-279): entity set-up, ticks, state/neighbour/entity exports.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _capi
from ._capi import (HEADING_ROAD_MASK, HEADING_TO_END, NO_NEIGHBOUR, PLACE_ROAD_START,  # noqa: F401
                    PLACE_UNIFORM_FRACTION, RNG_PCG32, RNG_XORSHIFT128, MsimError, check, lib)

__all__ = ["RoadMap", "Simulation", "MsimError", "set_device", "ENTITY_DTYPE", "RNG_XORSHIFT128", "RNG_PCG32",
           "HEADING_TO_END", "HEADING_ROAD_MASK", "NO_NEIGHBOUR", "lib"]

# Entity.hpp:33-46 (64-byte packed record)
ENTITY_DTYPE = np.dtype([("color", "<f4", (4,)), ("randomState", "<u4", (4,)), ("pos", "<f4", (2,)),
                         ("target", "<f4", (2,)), ("direction", "<f4", (2,)), ("roadIndex", "<u4"),
                         ("initialized", "<u4")])
assert ENTITY_DTYPE.itemsize == 64

# GpuQuadTree.hpp:14-41 (64-byte node) and :44-62 (20-byte entity link)
NODE_DTYPE = np.dtype([("acquireLock", "<i4"), ("writeLock", "<i4"), ("readerLock", "<i4"), ("offsetX", "<f4"),
                       ("offsetY", "<f4"), ("width", "<f4"), ("height", "<f4"), ("contentType", "<u4"),
                       ("entityCount", "<u4"), ("first", "<u4"), ("prevNodeIndex", "<u4"), ("nextTL", "<u4"),
                       ("nextTR", "<u4"), ("nextBL", "<u4"), ("nextBR", "<u4"), ("padding", "<u4")])
LINK_DTYPE = np.dtype([("nodeIndex", "<u4"), ("typeNext", "<u4"), ("next", "<u4"), ("typePrev", "<u4"),
                       ("prev", "<u4")])
assert NODE_DTYPE.itemsize == 64 and LINK_DTYPE.itemsize == 20
QUAD_TREE_MAX_DEPTH = 8        # Simulator.hpp:36
QUAD_TREE_ENTITY_NODE_CAP = 10  # Simulator.hpp:37


def node_count(max_depth: int) -> int:
    """GpuQuadTree.cpp:12-18 calc_node_count."""
    return sum(4 ** i for i in range(max_depth))


def build_quad_tree(pos, width: float, height: float, max_depth: int = QUAD_TREE_MAX_DEPTH,
                    node_cap: int = QUAD_TREE_ENTITY_NODE_CAP):
    """Reference-layout quad tree of host positions (id-order insertion)."""
    pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 2)
    nodes = np.zeros(node_count(max_depth), NODE_DTYPE)
    links = np.zeros(pos.shape[0], LINK_DTYPE)
    used = ctypes.c_uint32()
    check(lib().msim_quad_tree_build(_ptr(pos, ctypes.c_float), pos.shape[0], width, height, max_depth, node_cap,
                                     nodes.ctypes.data_as(ctypes.c_void_p), nodes.shape[0],
                                     links.ctypes.data_as(ctypes.c_void_p), ctypes.byref(used)))
    return nodes, links, used.value


_RNG_KINDS = {"xorshift128": RNG_XORSHIFT128, "pcg32": RNG_PCG32}


def set_device(device: int) -> None:
    """The GPU that contexts created by this thread from now on use (msim_set_device);
    the library's CUDA runtime does not follow torch.cuda.set_device."""
    check(lib().msim_set_device(int(device)))


def _ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype)) if a is not None else None


@dataclass
class RoadMap:
    """Road graph: road_pos (R,4) float32 start.x, start.y, end.x, end.y; road_conn (R,4)
    uint32 connIndexStart, connCountStart, connIndexEnd, connCountEnd; connections (C,)
    uint32 (connectionRoadIndexList); width/height = maxDistLat/maxDistLong."""

    road_pos: np.ndarray
    road_conn: np.ndarray
    connections: np.ndarray
    width: float
    height: float

    def __post_init__(self):
        self.road_pos = np.ascontiguousarray(self.road_pos, dtype=np.float32).reshape(-1, 4)
        self.road_conn = np.ascontiguousarray(self.road_conn, dtype=np.uint32).reshape(-1, 4)
        self.connections = np.ascontiguousarray(self.connections, dtype=np.uint32).reshape(-1)
        self.width = float(np.float32(self.width))
        self.height = float(np.float32(self.height))

    @property
    def num_roads(self) -> int:
        return int(self.road_pos.shape[0])

    def view(self) -> _capi.MsimMap:
        m = _capi.MsimMap()
        m.num_roads = self.num_roads
        m.num_connections = int(self.connections.shape[0])
        m.road_pos = _ptr(self.road_pos, ctypes.c_float)
        m.road_conn = _ptr(self.road_conn, ctypes.c_uint32)
        m.connections = _ptr(self.connections, ctypes.c_uint32)
        m.width = self.width
        m.height = self.height
        return m

    @classmethod
    def _from_buf(cls, buf: ctypes.c_void_p) -> "RoadMap":
        try:
            v = _capi.MsimMap()
            check(lib().msim_map_view(buf, ctypes.byref(v)))
            R, C = v.num_roads, v.num_connections
            pos = np.ctypeslib.as_array(v.road_pos, shape=(max(R, 1) * 4,))[: R * 4].copy() if R else np.zeros(0)
            conn = np.ctypeslib.as_array(v.road_conn, shape=(max(R, 1) * 4,))[: R * 4].copy() if R else np.zeros(0)
            cl = np.ctypeslib.as_array(v.connections, shape=(C,)).copy() if C else np.zeros(0, np.uint32)
            return cls(pos, conn, cl, v.width, v.height)
        finally:
            lib().msim_map_free(buf)

    @classmethod
    def load_json(cls, path: str) -> "RoadMap":
        """Map::load_from_file (Map.cpp:28-150)."""
        buf = ctypes.c_void_p()
        check(lib().msim_map_load_json(str(path).encode(), ctypes.byref(buf)))
        return cls._from_buf(buf)

    @classmethod
    def lattice(cls, side: int, seed: int, spacing: float = 50.0, jitter: float = 10.0,
                keep_prob: float = 0.9) -> "RoadMap":
        """Synthetic side x side intersection lattice in the reference map format."""
        buf = ctypes.c_void_p()
        check(lib().msim_map_generate_lattice(side, seed, spacing, jitter, keep_prob, ctypes.byref(buf)))
        return cls._from_buf(buf)

    def write_json(self, path: str) -> None:
        v = self.view()
        check(lib().msim_map_write_json(ctypes.byref(v), str(path).encode()))

    def validate(self) -> None:
        v = self.view()
        check(lib().msim_map_validate(ctypes.byref(v)))


class Simulation:
    """One simulation context on the current CUDA device.

    Reference mode (random_move.comp as written): rng="xorshift128", dt=1.0,
    speeds 1.4 (init_entities(speed=(1.4, 1.4))), radius 10.
    """

    def __init__(self, road_map: RoadMap, num_entities: int, *, rng: str = "xorshift128", dt: float = 1.0,
                 radius: float = 10.0, cap: int = 64, cell_size: float = 0.0, resort_interval: int = 0,
                 index: str = "auto", reuse: bool = True):
        self.map = road_map
        self.n = int(num_entities)
        self.cap = int(cap)
        self.rng_kind = _RNG_KINDS[rng]
        p = _capi.MsimParams(num_entities=self.n, rng_kind=self.rng_kind, dt=dt, radius=radius, cap=self.cap,
                             cell_size=cell_size, resort_interval=resort_interval,
                             flags={"auto": 0, "full": _capi.PARAM_FULL_SORT,
                                    "incremental": _capi.PARAM_INCREMENTAL}[index]
                             | (0 if reuse else _capi.PARAM_NO_REUSE))
        self._ctx = ctypes.c_void_p()
        v = road_map.view()
        check(lib().msim_create(ctypes.byref(v), ctypes.byref(p), ctypes.byref(self._ctx)))

    # -- lifecycle ---------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_ctx", None) is not None and self._ctx.value:
            lib().msim_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- entities ----------------------------------------------------------
    def init_entities(self, seed: int, placement: str = "start", speed=(1.4, 1.4)) -> None:
        pl = {"start": PLACE_ROAD_START, "fraction": PLACE_UNIFORM_FRACTION}[placement]
        ini = _capi.MsimInit(seed=seed, placement=pl, speed_min=speed[0], speed_max=speed[1])
        check(lib().msim_init_entities(self._ctx, ctypes.byref(ini)))

    def set_entities(self, pos, heading, rng, speed=None) -> None:
        pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(self.n, 2)
        heading = np.ascontiguousarray(heading, dtype=np.uint32).reshape(self.n)
        rng = np.ascontiguousarray(rng, dtype=np.uint32).reshape(self.n, 4)
        if speed is not None:
            speed = np.ascontiguousarray(speed, dtype=np.float32).reshape(self.n)
        check(lib().msim_set_entities(self._ctx, _ptr(pos, ctypes.c_float), _ptr(heading, ctypes.c_uint32),
                                      _ptr(rng, ctypes.c_uint32), _ptr(speed, ctypes.c_float)))

    def set_road_factors(self, factors) -> None:
        f = np.ascontiguousarray(factors, dtype=np.float32).reshape(self.map.num_roads)
        check(lib().msim_set_road_factors(self._ctx, _ptr(f, ctypes.c_float)))

    # -- ticks ---------------------------------------------------------------
    def step(self, ticks: int = 1, neighbours: bool = False) -> None:
        check(lib().msim_step(self._ctx, ticks, _capi.STEP_NEIGHBOURS if neighbours else 0))

    def sync(self) -> None:
        check(lib().msim_sync(self._ctx))

    def tick_host(self, state: dict, neighbours: bool = True, out: dict | None = None, with_idx: bool = False):
        """One tick with the state on the host (msim_tick_host): uploads state (pos,
        heading, rng, optional speed), moves, [index + query], returns the moved state
        and, with neighbours, the counts (and lists when with_idx).  `out` may supply
        the output arrays (page-locked ones let the copies overlap)."""
        n = self.n
        pos = np.ascontiguousarray(state["pos"], dtype=np.float32).reshape(n, 2)
        head = np.ascontiguousarray(state["heading"], dtype=np.uint32).reshape(n)
        rng = np.ascontiguousarray(state["rng"], dtype=np.uint32).reshape(n, 4)
        speed = state.get("speed")
        if speed is not None:
            speed = np.ascontiguousarray(speed, dtype=np.float32).reshape(n)
        if out is None:
            out = {"pos": np.empty((n, 2), np.float32), "heading": np.empty(n, np.uint32),
                   "rng": np.empty((n, 4), np.uint32)}
            if neighbours:
                out["count"] = np.empty(n, np.uint32)
                if with_idx and self.cap:
                    out["idx"] = np.empty((n, self.cap), np.uint32)
        check(lib().msim_tick_host(self._ctx, _ptr(pos, ctypes.c_float), _ptr(head, ctypes.c_uint32),
                                   _ptr(rng, ctypes.c_uint32), _ptr(speed, ctypes.c_float),
                                   _capi.STEP_NEIGHBOURS if neighbours else 0, _ptr(out.get("pos"), ctypes.c_float),
                                   _ptr(out.get("heading"), ctypes.c_uint32), _ptr(out.get("rng"), ctypes.c_uint32),
                                   _ptr(out.get("count"), ctypes.c_uint32), _ptr(out.get("idx"), ctypes.c_uint32)))
        return out

    @property
    def tick(self) -> int:
        t = ctypes.c_uint64()
        check(lib().msim_get_tick(self._ctx, ctypes.byref(t)))
        return t.value

    # -- exports ---------------------------------------------------------------
    def get_state(self, out=None):
        """dict of pos (N,2) f32, heading (N,) u32, rng (N,4) u32, speed (N,) f32, by entity id."""
        if out is None:
            out = {"pos": np.empty((self.n, 2), np.float32), "heading": np.empty(self.n, np.uint32),
                   "rng": np.empty((self.n, 4), np.uint32), "speed": np.empty(self.n, np.float32)}
        check(lib().msim_get_state(self._ctx, _ptr(out.get("pos"), ctypes.c_float),
                                   _ptr(out.get("heading"), ctypes.c_uint32), _ptr(out.get("rng"), ctypes.c_uint32),
                                   _ptr(out.get("speed"), ctypes.c_float)))
        return out

    def get_neighbours(self, with_idx: bool = True, out=None):
        """(count (N,), idx (N, cap) or None) of the last neighbour tick; `out` = a
        (count, idx) pair of arrays to fill instead of new ones."""
        if out is not None:
            count, idx = out
            if count.dtype != np.uint32 or count.shape != (self.n,) or not count.flags.c_contiguous:
                raise ValueError("out count must be a contiguous uint32 array of num_entities")
            if not (with_idx and self.cap):
                idx = None
            elif idx.dtype != np.uint32 or idx.shape != (self.n, self.cap) or not idx.flags.c_contiguous:
                raise ValueError("out idx must be a contiguous uint32 array of (num_entities, cap)")
        else:
            count = np.empty(self.n, np.uint32)
            idx = np.empty((self.n, self.cap), np.uint32) if (with_idx and self.cap) else None
        check(lib().msim_get_neighbours(self._ctx, _ptr(count, ctypes.c_uint32), _ptr(idx, ctypes.c_uint32)))
        return count, idx

    def collision_pairs(self) -> int:
        v = ctypes.c_uint64()
        check(lib().msim_get_collision_pairs(self._ctx, ctypes.byref(v)))
        return v.value

    def export_entities(self) -> np.ndarray:
        out = np.empty(self.n, ENTITY_DTYPE)
        check(lib().msim_export_entities_aos(self._ctx, out.ctypes.data_as(ctypes.c_void_p), self.n))
        return out

    def export_quad_tree(self, max_depth: int = QUAD_TREE_MAX_DEPTH, node_cap: int = QUAD_TREE_ENTITY_NODE_CAP):
        """Simulator::get_quad_tree_nodes: (nodes, links, nodes_used) in the reference layout."""
        nodes = np.zeros(node_count(max_depth), NODE_DTYPE)
        links = np.zeros(self.n, LINK_DTYPE)
        used = ctypes.c_uint32()
        check(lib().msim_export_quad_tree(self._ctx, max_depth, node_cap, nodes.ctypes.data_as(ctypes.c_void_p),
                                          nodes.shape[0], links.ctypes.data_as(ctypes.c_void_p), ctypes.byref(used)))
        return nodes, links, used.value

    # -- reports / timing ------------------------------------------------------
    def info(self) -> dict:
        i = _capi.MsimInfo()
        check(lib().msim_get_info(self._ctx, ctypes.byref(i)))
        return {f: getattr(i, f) for f, _ in _capi.MsimInfo._fields_}

    def launch_count(self) -> int:
        v = ctypes.c_uint64()
        check(lib().msim_get_launch_count(self._ctx, ctypes.byref(v)))
        return v.value

    def save_state(self, path) -> None:
        """Snapshot of the entity state and tick counter (msim_save_state)."""
        check(lib().msim_save_state(self._ctx, str(path).encode()))

    def load_state(self, path) -> None:
        """Resume from a snapshot written for the same configuration (msim_load_state)."""
        check(lib().msim_load_state(self._ctx, str(path).encode()))

    def set_wait_limit(self, polls: int) -> None:
        """Polls before a bounded device wait of the index gives up (0: the default)."""
        check(lib().msim_set_wait_limit(self._ctx, polls))

    def inject_fault(self, fault: int, arg: int = 0) -> None:
        """Arms one host-side fault (msim_debug.h: FAULT_SORT_TILE, FAULT_LAUNCH)."""
        check(lib().msim_debug_inject(self._ctx, fault, arg))

    def set_profiling(self, on: bool) -> None:
        check(lib().msim_set_profiling(self._ctx, 1 if on else 0))

    def reset_kernel_stats(self) -> None:
        check(lib().msim_reset_kernel_stats(self._ctx))

    def kernel_stats(self) -> dict:
        out = {}
        for k in range(lib().msim_kernel_count()):
            n = ctypes.c_uint64()
            ms = ctypes.c_double()
            check(lib().msim_get_kernel_stats(self._ctx, k, ctypes.byref(n), ctypes.byref(ms)))
            if n.value:
                out[lib().msim_kernel_name(k).decode()] = {"launches": n.value, "ms": ms.value}
        return out

    def sort_stats(self) -> dict:
        """Index updates since the stats were reset and the entries their radix passes sorted."""
        u, e = ctypes.c_uint64(), ctypes.c_uint64()
        check(lib().msim_get_sort_stats(self._ctx, ctypes.byref(u), ctypes.byref(e)))
        return {"index_updates": u.value, "sorted_entries": e.value}

    def host_tick_stats(self) -> dict:
        """Host ticks since the stats were reset, those whose query read the previous
        state's index with widened boxes, and the last measured displacement."""
        h, s, d = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_float()
        check(lib().msim_get_host_tick_stats(self._ctx, ctypes.byref(h), ctypes.byref(s), ctypes.byref(d)))
        return {"host_ticks": h.value, "skin_queries": s.value, "last_displacement": d.value}

    def timer_begin(self) -> None:
        check(lib().msim_timer_begin(self._ctx))

    def timer_end(self) -> float:
        ms = ctypes.c_float()
        check(lib().msim_timer_end(self._ctx, ctypes.byref(ms)))
        return ms.value


def ensemble_config(count: int = 512, seed: int = 20261203, side_range=(16, 256), entity_range=(1_000, 200_000)):
    """Instance sizes of the batched ensemble: lattice side uniform in side_range
    (inclusive), entity count log-uniform in entity_range, instance seed = index +
    seed.  Drawn with numpy's PCG64 generator seeded by `seed`."""
    rs = np.random.default_rng(seed)
    sides = rs.integers(side_range[0], side_range[1] + 1, count)
    lo, hi = np.log(entity_range[0]), np.log(entity_range[1])
    entities = np.floor(np.exp(rs.uniform(lo, hi, count))).astype(np.int64)
    seeds = np.arange(count, dtype=np.int64) + seed
    return [int(x) for x in sides], [int(x) for x in entities], [int(x) for x in seeds]


class Batch:
    """Batched ensemble: independent instances (map, entity count, init) advanced by
    one persistent launch per msim_batch_step call (move ticks only)."""

    def __init__(self, maps, num_entities, *, rng: str = "pcg32", dt: float = 0.1):
        self.maps = list(maps)
        self.n = [int(x) for x in num_entities]
        views = (_capi.MsimMap * len(self.maps))(*[m.view() for m in self.maps])
        counts = np.ascontiguousarray(self.n, dtype=np.uint32)
        self._b = ctypes.c_void_p()
        check(lib().msim_batch_create(views, _ptr(counts, ctypes.c_uint32), len(self.maps), _RNG_KINDS[rng], dt,
                                      ctypes.byref(self._b)))

    def close(self):
        if getattr(self, "_b", None) is not None and self._b.value:
            lib().msim_batch_destroy(self._b)
            self._b = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def init_entities(self, seeds, placement: str = "fraction", speed=(1.0, 1.6)):
        pl = {"start": PLACE_ROAD_START, "fraction": PLACE_UNIFORM_FRACTION}[placement]
        inits = (_capi.MsimInit * len(self.maps))(*[_capi.MsimInit(seed=int(s), placement=pl, speed_min=speed[0],
                                                                  speed_max=speed[1]) for s in seeds])
        check(lib().msim_batch_init_entities(self._b, inits))

    def step(self, ticks: int):
        check(lib().msim_batch_step(self._b, ticks))

    def sync(self):
        check(lib().msim_batch_sync(self._b))

    def get_state(self, instance: int):
        n = self.n[instance]
        out = {"pos": np.empty((n, 2), np.float32), "heading": np.empty(n, np.uint32),
               "rng": np.empty((n, 4), np.uint32), "speed": np.empty(n, np.float32)}
        check(lib().msim_batch_get_state(self._b, instance, _ptr(out["pos"], ctypes.c_float),
                                         _ptr(out["heading"], ctypes.c_uint32), _ptr(out["rng"], ctypes.c_uint32),
                                         _ptr(out["speed"], ctypes.c_float)))
        return out

    def schedule(self) -> dict:
        s = _capi.MsimBatchSchedule()
        check(lib().msim_batch_get_schedule(self._b, ctypes.byref(s)))
        c = s.num_classes
        return {"block_threads": s.block_threads, "class_min_entities": list(s.class_min_entities[:c]),
                "entities_per_thread": list(s.entities_per_thread[:c]), "tile_entities": list(s.tile_entities[:c])}

    def set_schedule(self, block_threads, class_min_entities, entities_per_thread, tile_entities):
        s = _capi.MsimBatchSchedule()
        s.block_threads = block_threads
        s.num_classes = len(class_min_entities)
        for i, (a, b, c) in enumerate(zip(class_min_entities, entities_per_thread, tile_entities)):
            s.class_min_entities[i], s.entities_per_thread[i], s.tile_entities[i] = a, b, c
        check(lib().msim_batch_set_schedule(self._b, ctypes.byref(s)))

    def tune(self, ticks: int, cache_path=None):
        check(lib().msim_batch_tune(self._b, ticks, str(cache_path).encode() if cache_path else None))

    def timer_begin(self):
        check(lib().msim_batch_timer_begin(self._b))

    def timer_end(self) -> float:
        ms = ctypes.c_float()
        check(lib().msim_batch_timer_end(self._b, ctypes.byref(ms)))
        return ms.value

    def info(self) -> dict:
        t, w, l = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint64()
        check(lib().msim_batch_info(self._b, ctypes.byref(t), ctypes.byref(w), ctypes.byref(l)))
        return {"total_entities": t.value, "work_items": w.value, "launches": l.value}


class PinnedBuffer:
    """Page-locked host memory (cudaMallocHost) viewed as a numpy array."""

    def __init__(self, shape, dtype):
        self.dtype = np.dtype(dtype)
        self.shape = tuple(shape) if isinstance(shape, (tuple, list)) else (int(shape),)
        nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        self._p = ctypes.c_void_p()
        check(lib().msim_host_alloc(max(nbytes, 1), ctypes.byref(self._p)))
        buf = (ctypes.c_char * max(nbytes, 1)).from_address(self._p.value)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=int(np.prod(self.shape))).reshape(self.shape)

    def free(self):
        if self._p.value:
            self.array = None
            lib().msim_host_free(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
