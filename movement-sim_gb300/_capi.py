"""ctypes declarations of the C ABI in include/msim.h (libmsim.so, built in place).

There is no fallback: importing the bindings without a built libmsim.so raises.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libmsim.so"

c_u32 = ctypes.c_uint32
c_u64 = ctypes.c_uint64
c_f32 = ctypes.c_float
u32p = ctypes.POINTER(ctypes.c_uint32)
f32p = ctypes.POINTER(ctypes.c_float)
vp = ctypes.c_void_p

MSIM_OK = 0
ERR_NAMES = {1: "MSIM_ERR_INVALID", 2: "MSIM_ERR_OOB", 3: "MSIM_ERR_CUDA", 4: "MSIM_ERR_TIMEOUT",
             5: "MSIM_ERR_NOMEM", 6: "MSIM_ERR_IO"}
RNG_XORSHIFT128 = 0
RNG_PCG32 = 1
HEADING_TO_END = 0x80000000
HEADING_ROAD_MASK = 0x7FFFFFFF
PLACE_ROAD_START = 0
PLACE_UNIFORM_FRACTION = 1
STEP_NEIGHBOURS = 1
PARAM_FULL_SORT = 1
PARAM_INCREMENTAL = 2
PARAM_NO_REUSE = 4
NO_NEIGHBOUR = 0xFFFFFFFF
FAULT_NONE = 0
FAULT_SORT_TILE = 1
FAULT_LAUNCH = 2


class MsimError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{ERR_NAMES.get(code, code)}: {message}")
        self.code = code


class MsimMap(ctypes.Structure):
    _fields_ = [("num_roads", c_u32), ("num_connections", c_u32), ("road_pos", f32p), ("road_conn", u32p),
                ("connections", u32p), ("width", c_f32), ("height", c_f32)]


class MsimParams(ctypes.Structure):
    _fields_ = [("num_entities", c_u32), ("rng_kind", c_u32), ("dt", c_f32), ("radius", c_f32), ("cap", c_u32),
                ("cell_size", c_f32), ("resort_interval", c_u32), ("flags", c_u32)]


class MsimInit(ctypes.Structure):
    _fields_ = [("seed", c_u64), ("placement", c_u32), ("speed_min", c_f32), ("speed_max", c_f32)]


class MsimBatchSchedule(ctypes.Structure):
    _fields_ = [("block_threads", c_u32), ("num_classes", c_u32), ("class_min_entities", c_u32 * 4),
                ("entities_per_thread", c_u32 * 4), ("tile_entities", c_u32 * 4)]


class MsimInfo(ctypes.Structure):
    _fields_ = [("num_entities", c_u32), ("num_roads", c_u32), ("num_connections", c_u32), ("tiles_x", c_u32),
                ("tiles_y", c_u32), ("key_bits", c_u32), ("sort_passes", c_u32), ("resort_interval", c_u32),
                ("cell_size", c_f32), ("cap", c_u32), ("device_bytes", c_u64)]


# name -> (restype, argtypes)
SIGNATURES = {
    "msim_last_error": (ctypes.c_char_p, []),
    "msim_version": (ctypes.c_char_p, []),
    "msim_map_load_json": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(vp)]),
    "msim_map_generate_lattice": (ctypes.c_int, [c_u32, c_u64, c_f32, c_f32, c_f32, ctypes.POINTER(vp)]),
    "msim_map_view": (ctypes.c_int, [vp, ctypes.POINTER(MsimMap)]),
    "msim_map_write_json": (ctypes.c_int, [ctypes.POINTER(MsimMap), ctypes.c_char_p]),
    "msim_map_validate": (ctypes.c_int, [ctypes.POINTER(MsimMap)]),
    "msim_map_free": (None, [vp]),
    "msim_set_wait_limit": (ctypes.c_int, [vp, c_u32]),
    "msim_set_device": (ctypes.c_int, [ctypes.c_int]),
    "msim_save_state": (ctypes.c_int, [vp, ctypes.c_char_p]),
    "msim_load_state": (ctypes.c_int, [vp, ctypes.c_char_p]),
    "msim_set_tick_timing": (ctypes.c_int, [vp, ctypes.c_int]),
    "msim_get_tick_times": (ctypes.c_int, [vp, f32p, f32p]),
    "msim_debug_inject": (ctypes.c_int, [vp, c_u32, c_u32]),
    "msim_debug_fail_device_alloc": (ctypes.c_int, [ctypes.c_int64]),
    "msim_create": (ctypes.c_int, [ctypes.POINTER(MsimMap), ctypes.POINTER(MsimParams), ctypes.POINTER(vp)]),
    "msim_destroy": (ctypes.c_int, [vp]),
    "msim_init_entities": (ctypes.c_int, [vp, ctypes.POINTER(MsimInit)]),
    "msim_set_entities": (ctypes.c_int, [vp, f32p, u32p, u32p, f32p]),
    "msim_set_road_factors": (ctypes.c_int, [vp, f32p]),
    "msim_step": (ctypes.c_int, [vp, c_u32, c_u32]),
    "msim_sync": (ctypes.c_int, [vp]),
    "msim_get_state": (ctypes.c_int, [vp, f32p, u32p, u32p, f32p]),
    "msim_get_neighbours": (ctypes.c_int, [vp, u32p, u32p]),
    "msim_get_collision_pairs": (ctypes.c_int, [vp, ctypes.POINTER(c_u64)]),
    "msim_export_entities_aos": (ctypes.c_int, [vp, vp, ctypes.c_size_t]),
    "msim_export_quad_tree": (ctypes.c_int, [vp, c_u32, c_u32, vp, c_u32, vp, u32p]),
    "msim_quad_tree_build": (ctypes.c_int, [f32p, c_u32, c_f32, c_f32, c_u32, c_u32, vp, c_u32, vp, u32p]),
    "msim_get_tick": (ctypes.c_int, [vp, ctypes.POINTER(c_u64)]),
    "msim_get_launch_count": (ctypes.c_int, [vp, ctypes.POINTER(c_u64)]),
    "msim_set_profiling": (ctypes.c_int, [vp, ctypes.c_int]),
    "msim_reset_kernel_stats": (ctypes.c_int, [vp]),
    "msim_get_kernel_stats": (ctypes.c_int, [vp, c_u32, ctypes.POINTER(c_u64), ctypes.POINTER(ctypes.c_double)]),
    "msim_get_sort_stats": (ctypes.c_int, [vp, ctypes.POINTER(c_u64), ctypes.POINTER(c_u64)]),
    "msim_get_host_tick_stats": (ctypes.c_int, [vp, ctypes.POINTER(c_u64), ctypes.POINTER(c_u64),
                                                ctypes.POINTER(ctypes.c_float)]),
    "msim_tick_host": (ctypes.c_int, [vp, f32p, u32p, u32p, f32p, c_u32, f32p, u32p, u32p, u32p, u32p]),
    "msim_kernel_count": (c_u32, []),
    "msim_kernel_name": (ctypes.c_char_p, [c_u32]),
    "msim_timer_begin": (ctypes.c_int, [vp]),
    "msim_timer_end": (ctypes.c_int, [vp, f32p]),
    "msim_host_alloc": (ctypes.c_int, [ctypes.c_size_t, ctypes.POINTER(vp)]),
    "msim_host_free": (ctypes.c_int, [vp]),
    "msim_get_info": (ctypes.c_int, [vp, ctypes.POINTER(MsimInfo)]),
    "msim_batch_default_schedule": (ctypes.c_int, [ctypes.POINTER(MsimBatchSchedule)]),
    "msim_batch_create": (ctypes.c_int, [ctypes.POINTER(MsimMap), u32p, c_u32, c_u32, c_f32, ctypes.POINTER(vp)]),
    "msim_batch_destroy": (ctypes.c_int, [vp]),
    "msim_batch_init_entities": (ctypes.c_int, [vp, ctypes.POINTER(MsimInit)]),
    "msim_batch_step": (ctypes.c_int, [vp, c_u32]),
    "msim_batch_sync": (ctypes.c_int, [vp]),
    "msim_batch_get_state": (ctypes.c_int, [vp, c_u32, f32p, u32p, u32p, f32p]),
    "msim_batch_set_schedule": (ctypes.c_int, [vp, ctypes.POINTER(MsimBatchSchedule)]),
    "msim_batch_get_schedule": (ctypes.c_int, [vp, ctypes.POINTER(MsimBatchSchedule)]),
    "msim_batch_tune": (ctypes.c_int, [vp, c_u32, ctypes.c_char_p]),
    "msim_batch_timer_begin": (ctypes.c_int, [vp]),
    "msim_batch_timer_end": (ctypes.c_int, [vp, f32p]),
    "msim_batch_info": (ctypes.c_int, [vp, ctypes.POINTER(c_u64), u32p, ctypes.POINTER(c_u64)]),
}

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is not built; run __graft_entry__.build() (needs nvcc)")
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(rc: int) -> None:
    if rc != MSIM_OK:
        raise MsimError(rc, lib().msim_last_error().decode(errors="replace"))
