"""Differentiable density calibration over the C ABI (msim_adj_*).

`Calibration` owns one adjoint context: a fixed road map, entities from the
deterministic initializer, a tick count, checkpoint interval and density grid.
`density_loss(calib, speed, factor, target)` is a torch.autograd.Function: its
forward runs the simulation and returns the MSE between the time-averaged
density and `target`; its backward returns d loss / d speed (per entity) and
d loss / d factor (per road) from the hand-written adjoint.  torch is used only
for device memory; every computation runs in libmsim.so.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _capi
from ._capi import check, lib

MODES = {"natural": 0, "record": 1, "replay": 2}
_RNG = {"xorshift128": 0, "pcg32": 1}


class MsimAdjParams(ctypes.Structure):
    _fields_ = [("num_entities", ctypes.c_uint32), ("rng_kind", ctypes.c_uint32), ("dt", ctypes.c_float),
                ("ticks", ctypes.c_uint32), ("checkpoint_interval", ctypes.c_uint32), ("grid_w", ctypes.c_uint32),
                ("grid_h", ctypes.c_uint32), ("placement", ctypes.c_uint32), ("seed", ctypes.c_uint64),
                ("speed_min", ctypes.c_float), ("speed_max", ctypes.c_float)]


_SIGS = {
    "msim_adj_create": (ctypes.c_int, [ctypes.POINTER(_capi.MsimMap), ctypes.POINTER(MsimAdjParams),
                                       ctypes.POINTER(ctypes.c_void_p)]),
    "msim_adj_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "msim_adj_get_initial_state": (ctypes.c_int, [ctypes.c_void_p, _capi.f32p, _capi.u32p, _capi.u32p, _capi.f32p]),
    "msim_adj_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_double)]),
    "msim_adj_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "msim_adj_get_gradients_f64": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                                  ctypes.POINTER(ctypes.c_double)]),
    "msim_adj_get_schedule": (ctypes.c_int, [ctypes.c_void_p, _capi.u32p]),
    "msim_adj_timer_begin": (ctypes.c_int, [ctypes.c_void_p]),
    "msim_adj_timer_end": (ctypes.c_int, [ctypes.c_void_p, _capi.f32p]),
    "msim_adj_phase_times": (ctypes.c_int, [ctypes.c_void_p, _capi.f32p]),
}
_bound = False


def _lib():
    global _bound
    L = lib()
    if not _bound:
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _bound = True
    return L


def _dptr(t, n, name):
    """Device pointer of a contiguous float32 CUDA tensor with n elements, or None."""
    if t is None:
        return None
    if not t.is_cuda or t.dtype.itemsize != 4 or not t.is_contiguous() or t.numel() != n:
        raise ValueError(f"{name} must be a contiguous 4-byte CUDA tensor with {n} elements")
    return ctypes.c_void_p(t.data_ptr())


class Calibration:
    def __init__(self, road_map, num_entities: int, ticks: int, *, dt: float = 0.1, rng: str = "pcg32",
                 checkpoint_interval: int = 100, grid=(512, 512), seed: int = 20261203, placement: str = "fraction",
                 speed=(1.0, 1.6)):
        self.map = road_map
        self.n = int(num_entities)
        self.ticks = int(ticks)
        self.grid = (int(grid[0]), int(grid[1]))
        p = MsimAdjParams(num_entities=self.n, rng_kind=_RNG[rng], dt=dt, ticks=self.ticks,
                          checkpoint_interval=checkpoint_interval, grid_w=self.grid[0], grid_h=self.grid[1],
                          placement={"start": 0, "fraction": 1}[placement], seed=seed, speed_min=speed[0],
                          speed_max=speed[1])
        self._a = ctypes.c_void_p()
        v = road_map.view()
        check(_lib().msim_adj_create(ctypes.byref(v), ctypes.byref(p), ctypes.byref(self._a)))

    def close(self):
        if getattr(self, "_a", None) is not None and self._a.value:
            _lib().msim_adj_destroy(self._a)
            self._a = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def initial_state(self) -> dict:
        n = self.n
        out = {"pos": np.empty((n, 2), np.float32), "heading": np.empty(n, np.uint32),
               "rng": np.empty((n, 4), np.uint32), "speed": np.empty(n, np.float32)}
        check(_lib().msim_adj_get_initial_state(self._a, out["pos"].ctypes.data_as(_capi.f32p),
                                                out["heading"].ctypes.data_as(_capi.u32p),
                                                out["rng"].ctypes.data_as(_capi.u32p),
                                                out["speed"].ctypes.data_as(_capi.f32p)))
        return out

    def forward(self, speed=None, factor=None, target=None, density=None, mode: str = "natural") -> float:
        """Runs the forward; tensors are CUDA float32 (any may be None).  Returns the loss."""
        import torch

        G = self.grid[0] * self.grid[1]
        args = (_dptr(speed, self.n, "speed"), _dptr(factor, self.map.num_roads, "factor"),
                _dptr(target, G, "target"), _dptr(density, G, "density"))
        torch.cuda.synchronize()  # the context's stream reads what torch wrote
        loss = ctypes.c_double()
        check(_lib().msim_adj_forward(self._a, *args, MODES[mode], ctypes.byref(loss)))
        return loss.value

    def backward(self, grad_speed=None, grad_factor=None) -> None:
        import torch

        gs = _dptr(grad_speed, self.n, "grad_speed")
        gf = _dptr(grad_factor, self.map.num_roads, "grad_factor")
        torch.cuda.synchronize()
        check(_lib().msim_adj_backward(self._a, gs, gf))

    def gradients_f64(self):
        gs = np.empty(self.n, np.float64)
        gf = np.empty(self.map.num_roads, np.float64)
        check(_lib().msim_adj_get_gradients_f64(self._a, gs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                gf.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return gs, gf

    def schedule(self) -> np.ndarray:
        w = (self.ticks + 31) // 32
        out = np.empty((self.n, w), np.uint32)
        check(_lib().msim_adj_get_schedule(self._a, out.ctypes.data_as(_capi.u32p)))
        return out

    def timer_begin(self):
        check(_lib().msim_adj_timer_begin(self._a))

    def timer_end(self) -> float:
        ms = ctypes.c_float()
        check(_lib().msim_adj_timer_end(self._a, ctypes.byref(ms)))
        return ms.value

    def phase_times(self) -> dict:
        """Device ms of the last forward and backward: forward kernel, loss, backward
        segment sweeps, road-gradient reduction."""
        ms = np.zeros(4, np.float32)
        check(_lib().msim_adj_phase_times(self._a, ms.ctypes.data_as(_capi.f32p)))
        return dict(zip(("forward", "loss", "backward_sweeps", "road_reduction"), ms.tolist()))


def _function():
    import torch

    class DensityLoss(torch.autograd.Function):
        """loss = mean((D(speed, factor) - target)^2) with the adjoint as backward."""

        @staticmethod
        def forward(ctx, speed, factor, calib, target):
            speed = speed.detach().contiguous().float()
            factor = factor.detach().contiguous().float()
            loss = calib.forward(speed, factor, target.detach().contiguous().float())
            ctx.calib = calib
            return torch.tensor(loss, dtype=torch.float64, device=speed.device)

        @staticmethod
        def backward(ctx, grad_out):
            calib = ctx.calib
            gs = torch.empty(calib.n, dtype=torch.float32, device=grad_out.device)
            gf = torch.empty(calib.map.num_roads, dtype=torch.float32, device=grad_out.device)
            calib.backward(gs, gf)
            g = grad_out.to(torch.float32)
            return gs * g, gf * g, None, None

    return DensityLoss


_DENSITY_LOSS = None


def density_loss(calib: Calibration, speed, factor, target):
    """Differentiable loss (torch scalar, float64) of speeds and road factors."""
    global _DENSITY_LOSS
    if _DENSITY_LOSS is None:
        _DENSITY_LOSS = _function()
    return _DENSITY_LOSS.apply(speed, factor, calib, target)
