"""Python face of the serving API (lx_server_*): continuous batching of submitted requests.

A request is a parameter set, a step count, dielectric boxes and optionally one DFT flux
plane.  The native worker admits requests under a device-memory budget, steps every running
request in one batch, chunk by chunk, and retires each as soon as it has run its steps.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _ffi
from ._ffi import LuxumError, Params, Request, ServerConfig, ServerStats
from .sim import Sim, params

STATES = {0: "queued", 1: "running", 2: "done", 3: "failed", 4: "cancelled"}


class Server:
    def __init__(self, precision: int = _ffi.LX_PREC_FP32, chunk: int = 100, budget_bytes: float = 0.0,
                 max_running: int = 0, tune_steps: int | None = None, tune_table=None):
        self.lib = _ffi.lib()
        cfg = ServerConfig()
        self.lib.lx_server_config_init(C.byref(cfg))
        cfg.precision, cfg.chunk, cfg.budget_bytes, cfg.max_running = precision, chunk, budget_bytes, max_running
        if tune_steps is not None:
            cfg.tune_steps = tune_steps
        if tune_table:
            arr = (_ffi.TuneEntry * len(tune_table))()
            for q, e in enumerate(tune_table):
                for k, _ in _ffi.TuneEntry._fields_:
                    setattr(arr[q], k, int(e[k]))
            cfg.tune_table = C.cast(arr, C.POINTER(_ffi.TuneEntry))
            cfg.tune_entries = len(tune_table)
        self.precision = precision
        h = C.c_void_p()
        self._check(self.lib.lx_server_create(C.byref(cfg), C.byref(h)))
        self.h = h
        self.nfreq = {}

    def _check(self, st: int) -> None:
        if st:
            raise LuxumError(st, self.lib.lx_last_error(None).decode())

    def submit(self, p: Params | dict, steps: int, boxes: Sequence = (), dft: tuple | None = None,
               material: dict | None = None, material_scale: float = 1.0) -> int:
        """boxes: [(lo, hi, eps_r), ...]; dft: (axis, index, omega array, every);
        material: {E component: F array of its staggered extent} (Cb = dt/(eps0*(1+F*scale)))."""
        if isinstance(p, dict):
            p = params(**p)
        r = Request()
        self.lib.lx_request_init(C.byref(r))
        r.params = p
        r.steps = steps
        keep = []
        for c, F in (material or {}).items():
            a = np.ascontiguousarray(F, dtype=np.float64)
            keep.append(a)
            r.material[c] = a.ctypes.data_as(C.POINTER(C.c_double))
        r.material_scale = material_scale
        b = np.array([list(lo) + list(hi) for lo, hi, _ in boxes], dtype=np.int32).reshape(-1)
        e = np.array([eps for _, _, eps in boxes], dtype=np.float64)
        r.n_boxes = len(boxes)
        if len(boxes):
            r.boxes = b.ctypes.data_as(C.POINTER(C.c_int))
            r.box_eps = e.ctypes.data_as(C.POINTER(C.c_double))
        w = None
        if dft is not None:
            axis, index, omega, every = dft
            w = np.ascontiguousarray(omega, dtype=np.float64)
            r.dft_axis, r.dft_index, r.dft_every, r.nfreq = axis, index, every, w.size
            r.omega = w.ctypes.data_as(C.POINTER(C.c_double))
        rid = C.c_longlong()
        self._check(self.lib.lx_server_submit(self.h, C.byref(r), C.byref(rid)))  # copies the arrays
        self.nfreq[rid.value] = 0 if w is None else w.size
        return rid.value

    def state(self, rid: int) -> str:
        s = C.c_int()
        self._check(self.lib.lx_server_poll(self.h, rid, C.byref(s)))
        return STATES[s.value]

    def wait(self, rid: int, timeout: float = -1.0) -> str:
        s = C.c_int()
        self._check(self.lib.lx_server_wait(self.h, rid, timeout, C.byref(s)))
        return STATES[s.value]

    def cancel(self, rid: int) -> None:
        self._check(self.lib.lx_server_cancel(self.h, rid))

    def flux(self, rid: int) -> np.ndarray:
        out = np.empty(self.nfreq[rid])
        self._check(self.lib.lx_server_flux(self.h, rid, out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out

    def max_e2(self, rid: int) -> float:
        v = C.c_double()
        self._check(self.lib.lx_server_max_e2(self.h, rid, C.byref(v)))
        return v.value

    def times(self, rid: int) -> tuple:
        """(submitted, started, finished) in seconds since the server was created (-1: not yet)."""
        t = (C.c_double * 3)()
        self._check(self.lib.lx_server_times(self.h, rid, t))
        return tuple(t)

    def take(self, rid: int, p: Params) -> Sim:
        """The finished request's handle as a Sim (the caller owns it from now on)."""
        h = C.c_void_p()
        self._check(self.lib.lx_server_take(self.h, rid, C.byref(h)))
        self.nfreq.pop(rid, None)
        return Sim._adopt(h, p)

    def release(self, rid: int) -> None:
        self._check(self.lib.lx_server_release(self.h, rid))
        self.nfreq.pop(rid, None)

    def error(self, rid: int) -> str:
        return self.lib.lx_server_error(self.h, rid).decode()

    def stats(self) -> dict:
        st = ServerStats()
        self._check(self.lib.lx_server_stats_get(self.h, C.byref(st)))
        return {n: getattr(st, n) for n, _ in ServerStats._fields_}

    def tune_table(self) -> list:
        """The tile shapes the server picked per request class (lx_server_tune_table)."""
        from .sim import _read_table

        return _read_table(lambda e, cap, n: self.lib.lx_server_tune_table(self.h, e, cap, n), self._check)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.lx_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
