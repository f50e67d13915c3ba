"""ctypes wrapper of the oracle (test infrastructure only).

The oracle is a CPU restatement of Luxum's time-stepping path (luxum_oracle.c).  Only
tests/, __graft_entry__.smoke() and bench.py's CPU legs use it, as the checker.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from luxum_gb300._ffi import Params

from .build import build_oracle

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle()
        L = C.CDLL(str(path))
        P = C.POINTER
        for name, res, args in [
            ("ox_params_size", C.c_size_t, []),
            ("ox_create", C.c_int, [P(Params), P(C.c_void_p)]),
            ("ox_destroy", None, [C.c_void_p]),
            ("ox_field_shape", C.c_int, [C.c_void_p, C.c_int, P(C.c_int)]),
            ("ox_read_field", C.c_int, [C.c_void_p, C.c_int, P(C.c_double), C.c_size_t]),
            ("ox_write_field", C.c_int, [C.c_void_p, C.c_int, P(C.c_double), C.c_size_t]),
            ("ox_set_cb", C.c_int, [C.c_void_p, C.c_int, P(C.c_double), C.c_size_t]),
            ("ox_set_material", C.c_int, [C.c_void_p, C.c_int, P(C.c_double), C.c_size_t, C.c_double]),
            ("ox_set_eps_box", C.c_int, [C.c_void_p, P(C.c_int), P(C.c_int), C.c_double]),
            ("ox_profile", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, P(C.c_double), C.c_size_t]),
            ("ox_set_threads", None, [C.c_void_p, C.c_int]),
            ("ox_timestep", C.c_int, [C.c_void_p]),
            ("ox_max_e2", C.c_double, [C.c_void_p]),
            ("ox_set_probes", C.c_int, [C.c_void_p, P(C.c_int), C.c_int, C.c_int]),
            ("ox_read_probes", C.c_int, [C.c_void_p, P(C.c_double), C.c_size_t, P(C.c_int)]),
            ("ox_step", C.c_int, [C.c_void_p, C.c_int]),
            ("ox_add_dft_plane", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, P(C.c_double), C.c_int]),
            ("ox_read_dft", C.c_int, [C.c_void_p, C.c_int, P(C.c_double), C.c_size_t]),
            ("ox_append_raw", C.c_int, [C.c_void_p, C.c_int, C.c_char_p]),
        ]:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleError(RuntimeError):
    def __init__(self, status: int):
        super().__init__(f"oracle rejected the parameters (status {status})")
        self.status = status


class OracleSim:
    """CPU restatement of one reference driver run (maxwell::solve dispatch)."""

    def __init__(self, p: Params, threads: int = 1):
        self.L = lib()
        h = C.c_void_p()
        st = self.L.ox_create(C.byref(p), C.byref(h))
        if st:
            raise OracleError(st)
        self.h = h
        self._p = p
        self.L.ox_set_threads(h, threads)
        self._np = 0
        self._cap = 0

    def close(self):
        if self.h:
            self.L.ox_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shape(self, comp):
        s = (C.c_int * 3)()
        assert self.L.ox_field_shape(self.h, comp, s) == 0
        return (s[0], s[1], s[2])

    def field(self, comp):
        out = np.empty(self.shape(comp), dtype=np.float64)
        assert self.L.ox_read_field(self.h, comp, _dptr(out), out.size) == 0
        return out

    def set_field(self, comp, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert self.L.ox_write_field(self.h, comp, _dptr(a), a.size) == 0

    def append_raw(self, comp, path):
        """Appends the component's doubles to a file (the bytes of one snapshot dataset)."""
        assert self.L.ox_append_raw(self.h, comp, str(path).encode()) == 0

    def set_cb(self, comp, cb):
        cb = np.ascontiguousarray(cb, dtype=np.float64)
        assert self.L.ox_set_cb(self.h, comp, _dptr(cb), cb.size) == 0

    def set_material(self, comp, F, scale=1e6):
        F = np.ascontiguousarray(F, dtype=np.float64)
        assert self.L.ox_set_material(self.h, comp, _dptr(F), F.size, scale) == 0

    def set_eps_box(self, lo, hi, eps_r):
        assert self.L.ox_set_eps_box(self.h, (C.c_int * 3)(*lo), (C.c_int * 3)(*hi), eps_r) == 0

    def profile(self, which: int, dim: int, is_e: bool, n: int):
        out = np.empty(n, dtype=np.float64)
        assert self.L.ox_profile(self.h, which, dim, int(is_e), _dptr(out), n) == 0
        return out

    def step(self, n=1):
        assert self.L.ox_step(self.h, n) == 0

    @property
    def t(self):
        return self.L.ox_timestep(self.h)

    def max_e2(self):
        return self.L.ox_max_e2(self.h)

    def set_probes(self, ijk, capacity):
        a = np.ascontiguousarray(np.asarray(ijk, dtype=np.int32).reshape(-1, 3))
        assert self.L.ox_set_probes(self.h, a.ctypes.data_as(C.POINTER(C.c_int)), a.shape[0], capacity) == 0
        self._np = a.shape[0]
        self._cap = capacity

    def add_dft_plane(self, axis, index, omega, every=1):
        w = np.ascontiguousarray(omega, dtype=np.float64)
        i = self.L.ox_add_dft_plane(self.h, axis, index, w.size, _dptr(w), every)
        assert i >= 0
        N = (self._p.Nx, 1 if self._p.isPlanar else self._p.Ny, self._p.Nz)
        self._dft = getattr(self, "_dft", {})
        self._dft[i] = (w.size, N[1] if axis == 0 else N[0], N[1] if axis == 2 else N[2])
        return i

    def dft(self, plane):
        nf, na, nb = self._dft[plane]
        raw = np.empty((nf, 4, na, nb, 2))
        assert self.L.ox_read_dft(self.h, plane, _dptr(raw), raw.size) == 0
        return raw[..., 0] + 1j * raw[..., 1]

    def probes(self):
        out = np.zeros((max(self._cap, 1), max(self._np, 1), 6))
        rows = C.c_int()
        assert self.L.ox_read_probes(self.h, _dptr(out), out.size, C.byref(rows)) == 0
        return out[: rows.value, : self._np]
