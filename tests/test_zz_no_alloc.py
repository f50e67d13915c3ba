"""lx_sim_read_field_noalloc against lx_sim_read_field.

The no-allocation read is for callers that must not let the library allocate device memory
when they read a field (their GPU memory belongs to another allocator, or a cudaMalloc's
device-wide synchronisation would break their latency budget).  It must return exactly what
the allocating read returns, on two calls in a row (the static staging array keeps the last
call's contents), and reject components larger than its 1048576-value staging array.
This file is collected last so that a failure here does not hide the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def _read_noalloc(sim, comp):
    out = np.full(sim.shape(comp), np.nan)
    st = sim.lib.lx_sim_read_field_noalloc(sim.h, comp, out.ctypes.data_as(C.POINTER(C.c_double)), out.size)
    assert st == 0, sim.lib.lx_last_error(sim.h)
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_read_matches_read_field(engine, precision):
    from luxum_gb300 import Sim

    p, steps, boxes = cases.build("3d_pml_axis")
    p.precision = precision
    sim = Sim(p)
    for lo, hi, eps in boxes:
        sim.set_eps_box(lo, hi, eps)
    sim.set_snapshots(5, 1 << 6, lambda t, c, a: None)  # keeps |E|^2 on the device
    sim.step(21)
    sim.sync()
    for comp in range(7):
        ref = sim.field(comp)
        first = _read_noalloc(sim, comp)
        second = _read_noalloc(sim, comp)
        assert np.array_equal(first, ref), comp
        assert np.array_equal(second, ref), comp
        assert np.any(ref != 0), comp
    sim.close()


def test_noalloc_read_rejects_oversized_component(engine):
    from luxum_gb300 import Sim

    p = cases.make(isPlanar=0, Nx=110, Ny=100, Nz=100)  # Ex holds 109*100*100 > 1048576 values
    sim = Sim(p)
    out = np.empty(sim.shape(0))
    st = sim.lib.lx_sim_read_field_noalloc(sim.h, 0, out.ctypes.data_as(C.POINTER(C.c_double)), out.size)
    assert st == 1
    assert b"at most 1048576" in sim.lib.lx_last_error(sim.h)
    sim.close()
