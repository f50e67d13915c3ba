"""Python face of the engine: parameters, simulation handles, numpy views of the fields.

Mirrors the reference's objects: `params(...)`/`read_yaml(path)` stand for class reader
(reader.h:50-174, reader.cc:68-162), `Sim` for the grid/vfield/maxwell trio a driver builds
(grid.cc:58-95, maxwell.cc:60-148) and its time loop (maxwell.cc:157-174).  Field arrays
come back in the reference's staggered extents (field.cc:58-77), C order.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable

import numpy as np

from . import _ffi
from ._ffi import LuxumError, Params


def params(**kw) -> Params:
    """lx_params with the reference defaults, then `kw` applied (names as in reader.h)."""
    p = Params()
    _ffi.lib().lx_params_init(C.byref(p))
    names = {n for n, _ in Params._fields_}
    for k, v in kw.items():
        if k not in names:
            raise KeyError(f"unknown parameter {k!r}")
        setattr(p, k, v)
    return p


def device_bytes(p: Params) -> int:
    """Device memory a handle for p would hold after creation (host-only estimate)."""
    n = C.c_size_t()
    st = _ffi.lib().lx_params_device_bytes(C.byref(p), C.byref(n))
    if st:
        raise LuxumError(st, _ffi.lib().lx_last_error(None).decode())
    return n.value


def step_bytes(p: Params) -> float:
    """Compulsory device-memory bytes of one time step for p (host-only): every field read
    and written once, Cb read once, every stored CPML psi entry read and written once."""
    b = C.c_double()
    st = _ffi.lib().lx_params_step_bytes(C.byref(p), C.byref(b))
    if st:
        raise LuxumError(st, _ffi.lib().lx_last_error(None).decode())
    return b.value


def trim_device_memory() -> None:
    """Waits for the device and returns the memory pool's unused memory to the driver."""
    lib = _ffi.lib()
    st = lib.lx_trim_device_memory()
    if st:
        raise LuxumError(st, lib.lx_last_error(None).decode())


def field_shape(p: Params, comp: int) -> tuple:
    """Staggered extent of a component for parameters p (host only)."""
    shp = (C.c_int * 3)()
    st = _ffi.lib().lx_params_field_shape(C.byref(p), comp, shp)
    if st:
        raise LuxumError(st, _ffi.lib().lx_last_error(None).decode())
    return (shp[0], shp[1], shp[2])


def read_yaml(path: str) -> Params:
    """Parses a Luxum parameters.yaml (reader::readYAML + checkData)."""
    p = Params()
    st = _ffi.lib().lx_params_from_yaml(str(path).encode(), C.byref(p))
    if st:
        raise LuxumError(st, _ffi.lib().lx_last_error(None).decode())
    return p


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Sim:
    """One simulation on the current GPU (an lx_sim handle)."""

    def __init__(self, p: Params | dict):
        if isinstance(p, dict):
            p = params(**p)
        self.lib = _ffi.lib()
        self.p = p
        h = C.c_void_p()
        st = self.lib.lx_sim_create(C.byref(p), C.byref(h))
        if st:
            raise LuxumError(st, self.lib.lx_last_error(None).decode())
        self.h = h
        self._cb = None

    @classmethod
    def _adopt(cls, h: C.c_void_p, p: Params) -> "Sim":
        """Wraps a handle created elsewhere (a finished server request)."""
        self = cls.__new__(cls)
        self.lib = _ffi.lib()
        self.p = p
        self.h = h
        self._cb = None
        return self

    # -- lifecycle
    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.lx_sim_destroy(self.h)
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

    def _check(self, st: int) -> None:
        if st:
            raise LuxumError(st, self.lib.lx_last_error(self.h).decode())

    # -- queries
    def shape(self, comp: int) -> tuple[int, int, int]:
        s = (C.c_int * 3)()
        self._check(self.lib.lx_sim_field_shape(self.h, comp, s))
        return (s[0], s[1], s[2])

    @property
    def t(self) -> int:
        return self.lib.lx_sim_timestep(self.h)

    def tune_class(self) -> dict:
        """The handle's tile-shape class (planar, size_class, precision, slab_class)."""
        e = _ffi.TuneEntry()
        self._check(self.lib.lx_sim_tune_class(self.h, C.byref(e)))
        return {k: getattr(e, k) for k, _ in _ffi.TuneEntry._fields_ if k != "march"}

    def max_e2(self) -> float:
        v = C.c_double()
        self._check(self.lib.lx_sim_max_e2(self.h, C.byref(v)))
        return v.value

    def info(self) -> dict:
        i = _ffi.Info()
        self._check(self.lib.lx_sim_info(self.h, C.byref(i)))
        return {"cells": i.cells, "device_bytes": i.device_bytes, "psi_h_entries": i.psi_h_entries,
                "psi_e_entries": i.psi_e_entries, "slab": list(i.slab), "uniform": i.uniform,
                "field_bytes": i.field_bytes}

    def counters(self) -> tuple[int, int, int]:
        k, a, b = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._check(self.lib.lx_sim_counters(self.h, C.byref(k), C.byref(a), C.byref(b)))
        return k.value, a.value, b.value

    # -- fields
    def field(self, comp: int) -> np.ndarray:
        shp = self.shape(comp)
        out = np.empty(shp, dtype=np.float64)
        self._check(self.lib.lx_sim_read_field(self.h, comp, _dptr(out), out.size))
        return out

    def set_field(self, comp: int, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.shape != self.shape(comp):
            raise ValueError(f"shape {a.shape} != {self.shape(comp)}")
        self._check(self.lib.lx_sim_write_field(self.h, comp, _dptr(a), a.size))

    def set_cb(self, comp: int, cb: np.ndarray) -> None:
        cb = np.ascontiguousarray(cb, dtype=np.float64)
        self._check(self.lib.lx_sim_set_cb(self.h, comp, _dptr(cb), cb.size))

    def set_material(self, comp: int, F: np.ndarray, scale: float = 1e6) -> None:
        F = np.ascontiguousarray(F, dtype=np.float64)
        self._check(self.lib.lx_sim_set_material(self.h, comp, _dptr(F), F.size, scale))

    def set_eps_box(self, lo, hi, eps_r: float) -> None:
        self._check(self.lib.lx_sim_set_eps_box(self.h, (C.c_int * 3)(*lo), (C.c_int * 3)(*hi), eps_r))

    # -- stepping
    def step(self, n: int = 1) -> None:
        self._check(self.lib.lx_sim_step(self.h, n))

    def time_kernels(self, n: int) -> dict:
        """Mean device ms per launch of each kernel over an instrumented pass of n steps."""
        out = (C.c_double * 4)()
        self._check(self.lib.lx_sim_time_kernels(self.h, n, out))
        return {"prologue": out[0], "h_update": out[1], "e_update": out[2], "probes": out[3]}

    def sync(self) -> None:
        self._check(self.lib.lx_sim_sync(self.h))

    def reset(self) -> None:
        self._check(self.lib.lx_sim_reset(self.h))

    def set_stream(self, stream_handle: int | None) -> None:
        self._check(self.lib.lx_sim_set_stream(self.h, C.c_void_p(stream_handle or 0)))

    # -- probes / snapshots
    def set_probes(self, ijk, capacity: int) -> None:
        a = np.ascontiguousarray(np.asarray(ijk, dtype=np.int32).reshape(-1, 3))
        self._check(self.lib.lx_sim_set_probes(self.h, a.ctypes.data_as(C.POINTER(C.c_int)), a.shape[0], capacity))
        self._nprobes = a.shape[0]
        self._probe_cap = capacity

    def probes(self) -> np.ndarray:
        n = getattr(self, "_nprobes", 0)
        cap = getattr(self, "_probe_cap", 0)
        out = np.zeros((max(cap, 1), max(n, 1), 6), dtype=np.float64)
        rows = C.c_int()
        self._check(self.lib.lx_sim_read_probes(self.h, _dptr(out), out.size, C.byref(rows)))
        return out[: rows.value, :n]

    def add_dft_plane(self, axis: int, index: int, omega, every: int = 1) -> int:
        w = np.ascontiguousarray(omega, dtype=np.float64)
        i = C.c_int()
        self._check(self.lib.lx_sim_add_dft_plane(self.h, axis, index, w.size, _dptr(w), every, C.byref(i)))
        n = [self.shape(0), self.shape(1), self.shape(2)]
        N = (self.p.Nx, 1 if self.p.isPlanar else self.p.Ny, self.p.Nz)
        na = N[1] if axis == 0 else N[0]
        nb = N[1] if axis == 2 else N[2]
        self._dft = getattr(self, "_dft", {})
        self._dft[i.value] = (w.size, na, nb)
        return i.value

    def dft(self, plane: int) -> np.ndarray:
        """Complex accumulators [nfreq, 4, na, nb] of one DFT plane."""
        nf, na, nb = self._dft[plane]
        raw = np.empty((nf, 4, na, nb, 2))
        self._check(self.lib.lx_sim_read_dft(self.h, plane, _dptr(raw), raw.size))
        return raw[..., 0] + 1j * raw[..., 1]

    def dft_flux(self, plane: int) -> np.ndarray:
        nf = self._dft[plane][0]
        out = np.empty(nf)
        self._check(self.lib.lx_sim_dft_flux(self.h, plane, _dptr(out), nf))
        return out

    def set_snapshots(self, every: int, mask: int, fn: Callable[[int, int, np.ndarray], None] | None) -> None:
        """fn(t, comp, array) is called from the handle's writer thread with a copy."""
        if fn is None or every == 0:
            self._cb = None
            self._check(self.lib.lx_sim_set_snapshots(self.h, 0, 0, _ffi.SNAPSHOT_FN(), None))
            return

        def trampoline(user, t, comp, data, shape):
            shp = (shape[0], shape[1], shape[2])
            n = shp[0] * shp[1] * shp[2]
            arr = np.ctypeslib.as_array(data, shape=(n,)).reshape(shp).copy()
            fn(t, comp, arr)

        self._cb = _ffi.SNAPSHOT_FN(trampoline)
        self._check(self.lib.lx_sim_set_snapshots(self.h, every, mask, self._cb, None))

    def set_max_series(self, capacity: int) -> None:
        """Keep max|E|^2 of every monitored step on the device (up to capacity between reads)."""
        self._check(self.lib.lx_sim_set_max_series(self.h, capacity))
        self._series_cap = capacity

    def max_series(self):
        """(steps, max|E|^2) recorded since the last call; empties the series."""
        cap = max(getattr(self, "_series_cap", 0), 1)
        ts = np.empty(cap, dtype=np.int32)
        vs = np.empty(cap)
        rows = C.c_int()
        self._check(self.lib.lx_sim_read_max_series(self.h, ts.ctypes.data_as(C.POINTER(C.c_int)),
                                                     vs.ctypes.data_as(C.POINTER(C.c_double)), cap, C.byref(rows)))
        return ts[: rows.value].copy(), vs[: rows.value].copy()

    def save(self, path: str) -> None:
        """Checkpoint: the whole state into one HDF5 file (fields as in the snapshot files)."""
        self._check(self.lib.lx_sim_save(self.h, str(path).encode()))

    def load(self, path: str) -> None:
        """Resume from a checkpoint written by a handle with the same parameters and DFT planes."""
        self._check(self.lib.lx_sim_load(self.h, str(path).encode()))

    def set_hdf5_output(self, every: int, comp: int, path: str, first: int = 0) -> None:
        self._check(self.lib.lx_sim_set_hdf5_output(self.h, every, first, comp, str(path).encode()))


def hdf5_write(path: str, datasets: dict) -> None:
    """Writes {name: 3-D float64 array} (all of one shape) as an HDF5 file in fileio.cc's layout."""
    lib = _ffi.lib()
    names = list(datasets)
    arrs = [np.ascontiguousarray(datasets[n], dtype=np.float64) for n in names]
    shape = arrs[0].shape if arrs else (0, 0, 0)
    if any(a.shape != shape or a.ndim != 3 for a in arrs):
        raise ValueError("all datasets must be 3-D arrays of one shape")
    cnames = (C.c_char_p * len(names))(*[n.encode() for n in names])
    ptrs = (C.POINTER(C.c_double) * len(arrs))(*[_dptr(a) for a in arrs])
    st = lib.lx_hdf5_write(str(path).encode(), len(names), cnames, ptrs, (C.c_int * 3)(*shape))
    if st:
        raise LuxumError(st, lib.lx_last_error(None).decode())


def hdf5_read(path: str, dataset: str) -> np.ndarray:
    """Reads one float dataset (rank <= 3) of an HDF5 file; returns a 3-D array."""
    lib = _ffi.lib()
    shp = (C.c_int * 3)()
    st = lib.lx_hdf5_read(str(path).encode(), dataset.encode(), None, 0, shp)
    if st:
        raise LuxumError(st, lib.lx_last_error(None).decode())
    out = np.empty((shp[0], shp[1], shp[2]), dtype=np.float64)
    st = lib.lx_hdf5_read(str(path).encode(), dataset.encode(), _dptr(out), out.size, shp)
    if st:
        raise LuxumError(st, lib.lx_last_error(None).decode())
    return out


class Batch:
    """Many simulations stepped together (lx_batch_*): one launch per half step for all."""

    def __init__(self, chunk: int = 100):
        self.lib = _ffi.lib()
        h = C.c_void_p()
        st = self.lib.lx_batch_create(C.byref(h))
        if st:
            raise LuxumError(st, self.lib.lx_last_error(None).decode())
        self.h = h
        self.members = []
        self._check(self.lib.lx_batch_set_chunk(self.h, chunk))

    def _check(self, st: int) -> None:
        if st:
            raise LuxumError(st, self.lib.lx_last_error(None).decode())

    def add(self, sim: Sim) -> None:
        self._check(self.lib.lx_batch_add(self.h, sim.h))
        self.members.append(sim)

    def remove(self, sim: Sim) -> None:
        self._check(self.lib.lx_batch_remove(self.h, sim.h))
        self.members.remove(sim)

    def step(self, n: int) -> None:
        self._check(self.lib.lx_batch_step(self.h, n))

    def step_async(self, n: int) -> None:
        self._check(self.lib.lx_batch_step_async(self.h, n))

    def wait(self) -> None:
        self._check(self.lib.lx_batch_wait(self.h))

    def set_march(self, planar_rows: int, planes_3d: int) -> None:
        """Cells each thread of the batched kernels walks along x (1, 2, 4 or 8)."""
        self._check(self.lib.lx_batch_set_march(self.h, planar_rows, planes_3d))

    def march(self) -> tuple:
        a, b = C.c_int(), C.c_int()
        self._check(self.lib.lx_batch_get_march(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def autotune(self, steps: int = 20) -> tuple:
        """Times each march on twins of each class of member and records the fastest per class
        (tune_table); returns the per-dimension march (planar, 3-D), the largest class's pick."""
        a, b = C.c_int(), C.c_int()
        self._check(self.lib.lx_batch_autotune(self.h, steps, C.byref(a), C.byref(b)))
        return a.value, b.value

    def tune_member(self, sim, steps: int = 10) -> int:
        """Tunes the class of `sim` on twins of it; returns the pick (0: no tile shape)."""
        m = C.c_int()
        self._check(self.lib.lx_batch_tune_member(self.h, sim.h, steps, C.byref(m)))
        return m.value

    def tune_table(self) -> list:
        """The tile-shape table: dicts with planar, size_class, precision, slab_class, march."""
        return _read_table(lambda e, cap, n: self.lib.lx_batch_get_tune_table(self.h, e, cap, n), self._check)

    def set_tune_table(self, entries) -> None:
        arr = (_ffi.TuneEntry * max(len(entries), 1))()
        for q, e in enumerate(entries):
            for k, _ in _ffi.TuneEntry._fields_:
                setattr(arr[q], k, int(e[k]))
        self._check(self.lib.lx_batch_set_tune_table(self.h, arr, len(entries)))

    def __len__(self):
        return self.lib.lx_batch_size(self.h)

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.lx_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _read_table(get, check) -> list:
    """Reads a tile-shape table through get(entries, cap, byref(n))."""
    n = C.c_int()
    check(get(None, 0, C.byref(n)))
    arr = (_ffi.TuneEntry * max(n.value, 1))()
    check(get(arr, n.value, C.byref(n)))
    return [{k: getattr(arr[q], k) for k, _ in _ffi.TuneEntry._fields_} for q in range(n.value)]
