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


@pytest.mark.parametrize("precision", [0, 1, 2])
def test_noalloc_read_matches_read_field(engine, precision):
    """3-D handle in FP64, FP32 and FP16 storage (H stored scaled, read back unscaled)."""
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


@pytest.mark.parametrize("steps", [37, 38])
def test_noalloc_read_planar_two_buffer_state(engine, steps):
    """A planar FP32 handle stepped alone keeps its state in two buffers and, after an odd
    number of steps, in the second one: the read must pick the same buffer as the
    allocating read."""
    from luxum_gb300 import Sim

    p, _, boxes = cases.build("planar_pml_axis")
    p.precision = 1
    sim = Sim(p)
    for lo, hi, eps in boxes:
        sim.set_eps_box(lo, hi, eps)
    sim.step(steps)
    sim.sync()
    for comp in (1, 3, 5):  # Ey, Hx, Hz: the planar components
        ref = sim.field(comp)
        for _ in range(2):
            assert np.array_equal(_read_noalloc(sim, comp), ref), comp
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
