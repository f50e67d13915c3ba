"""Single-sweep steps (planar and 3-D) against the two-sweep kernels.

Handles with float compute (FP32 and FP16 storage) form H and E of a step in one launch
over two state buffers: state n is read from one and state n+1 written to the other.
Handles created while LUXUM_TWO_SWEEP=1 is set use the in-place two-sweep kernels instead.
Both must give the same fields, DFT accumulators, probe series and max|E|^2 series, bit for
bit: at odd and even step counts, through a checkpoint written at an odd step, and across
joining and leaving a batch (batches update their members in place).
"""
import os

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

OMEGA = 2 * np.pi * np.linspace(3e10, 1.5e11, 5)


def _big(precision, uniform=True):
    """A planar grid large enough for full 16-row warps and interior blocks: CPML 16, TF/SF
    box, a pulsed point source, a dielectric block."""
    kw = dict(isPlanar=1, Nx=300, Ny=1, Nz=520, **cases.pw((1, 0, 0), (0, 1, 0), ((24, 275), (0, 0), (24, 495))),
              **cases.pml(16), usePS=1, source_kind=1, Nx_source=150, Nz_source=260, amp_source=1.0,
              omega_source=2.0e11, src_t0=15.0, src_tw=6.0, precision=precision)
    if not uniform:
        kw["dz"] = 0.8e-3
    return cases.make(**kw), [((120, 0, 200), (180, 1, 330), 4.0)]


def _small(name, precision):
    p, _, boxes = cases.build(name)
    p.precision = precision
    return p, boxes


def _sim(p, boxes, dft=True):
    from luxum_gb300 import Sim

    s = Sim(p)
    for lo, hi, eps in boxes:
        s.set_eps_box(lo, hi, eps)
    if dft:
        s.add_dft_plane(0, p.Nx // 3, OMEGA)
        s.add_dft_plane(2, p.Nz // 2, OMEGA, every=3)  # z-normal: its first sampled component (Ex) is absent
    return s


def _pair(p, boxes, dft=True):
    """(single-sweep handle, two-sweep handle) of the same parameters."""
    os.environ.pop("LUXUM_TWO_SWEEP", None)
    os.environ["LUXUM_SWEEP3"] = "1"  # 3-D float handles too
    try:
        a = _sim(p, boxes, dft)
    finally:
        del os.environ["LUXUM_SWEEP3"]
    os.environ["LUXUM_TWO_SWEEP"] = "1"
    try:
        b = _sim(p, boxes, dft)
    finally:
        del os.environ["LUXUM_TWO_SWEEP"]
    # the single-sweep handle holds a second copy of the fields
    assert a.info()["device_bytes"] > b.info()["device_bytes"]
    return a, b


def _same(a, b):
    assert a.t == b.t
    for c in range(6):  # the planar grids hold Ey, Hx, Hz only
        if np.prod(a.shape(c)):
            assert np.array_equal(a.field(c), b.field(c)), (a.t, c)
    for plane in getattr(a, "_dft", {}):
        assert np.array_equal(a.dft(plane), b.dft(plane)), a.t
    assert a.max_e2() == b.max_e2()


@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("name", ["planar_pml_axis", "planar_oblique", "planar_pml_std_oblique", "3d_pml_axis",
                                  "3d_oblique", "3d_pml_y_amax", "3d_pml_point_cw", "3d_pml_pulse_nonuniform"])
def test_sweep_equals_two_sweep_small(engine, name, precision):
    a, b = _pair(*_small(name, precision))
    for n in (1, 36, 1, 2, 17):  # odd and even step counts
        a.step(n)
        b.step(n)
        _same(a, b)
    assert np.isfinite(a.max_e2()) and a.max_e2() > 0


@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("uniform", [True, False])
def test_sweep_equals_two_sweep_large(engine, precision, uniform):
    p, boxes = _big(precision, uniform)
    a, b = _pair(p, boxes)
    ijk = np.array([[150, 0, 260], [30, 0, 40], [200, 0, 500], [298, 0, 518]], dtype=np.int32)
    for s in (a, b):
        s.set_probes(ijk, 200)
        s.set_max_series(200)
    a.step(61)
    b.step(61)
    _same(a, b)
    a.step(40)
    b.step(40)
    _same(a, b)
    assert np.array_equal(a.probes(), b.probes())
    ta, va = a.max_series()
    tb, vb = b.max_series()
    assert np.array_equal(ta, tb) and np.array_equal(va, vb)


def test_sweep_write_field_and_reset(engine):
    """Values written at an odd step are the state whichever buffer the next step reads."""
    p, boxes = _big(1)
    a, b = _pair(p, boxes, dft=False)
    a.step(11)
    b.step(11)
    rng = np.random.default_rng(7)
    for c in (1, 3, 5):
        v = rng.standard_normal(a.shape(c)) * 1e-3
        a.set_field(c, v)
        b.set_field(c, v)
    a.step(9)
    b.step(9)
    _same(a, b)
    a.reset()
    b.reset()
    a.step(3)
    b.step(3)
    _same(a, b)


def test_sweep_checkpoint_at_odd_step(engine, tmp_path):
    p, boxes = _big(1)
    a, b = _pair(p, boxes)
    a.step(33)
    b.step(33)
    path = str(tmp_path / "odd.h5")
    a.save(path)
    c = _sim(p, boxes)
    c.load(path)
    assert c.t == 33
    for s in (a, b, c):
        s.step(24)
    _same(a, b)
    _same(c, b)


@pytest.mark.parametrize("precision", [1, 2])
def test_sweep_handles_in_a_batch(engine, precision):
    """Batches update their members in place: a single-sweep handle that joins at an odd step
    moves its state into buffer 0, and back into buffer t & 1 when it steps alone again."""
    from luxum_gb300 import Batch

    specs = [_small("planar_pml_axis", precision), _small("planar_oblique", precision), _big(precision)]
    pairs = [_pair(p, boxes) for p, boxes in specs]
    for k, (a, b) in enumerate(pairs):  # ping-pong steps before joining, odd and even counts
        a.step(3 + k)
        b.step(3 + k)
    batch = Batch(chunk=10)
    for a, _ in pairs:
        batch.add(a)
    pairs[1][0].step(3)  # a member steps alone between batch steps
    pairs[1][1].step(3)
    batch.step(36)  # graph replays and direct steps
    for _, b in pairs:
        b.step(36)
    for a, b in pairs:
        _same(a, b)
    batch.remove(pairs[0][0])  # leaves at an odd step count and steps alone again
    assert pairs[0][0].t % 2 == 1
    for a, b in pairs:
        a.step(6)
        b.step(6)
        _same(a, b)


def _big3(precision, uniform=True, n=(256, 128, 160)):
    """A 3-D grid with every tile kind of the 3-D sweep: interior tiles, tiles in the CPML
    slabs and on the TF/SF faces, partial tiles at the y and z ends, and (at the default
    size) 16 planes per block."""
    nx, ny, nz = n
    mx, my, mz = (min(20, v // 3) for v in n)  # TF/SF faces inside the 10-cell CPML
    kw = dict(isPlanar=0, Nx=nx, Ny=ny, Nz=nz,
              **cases.pw((1, 0, 0), (0, 0, 1), ((mx, nx - 1 - mx), (my, ny - 1 - my), (mz, nz - 1 - mz))),
              **cases.pml(10, kappa=5.0, a_max=0.05), usePS=1, source_kind=1, Nx_source=nx // 2, Ny_source=ny // 2,
              Nz_source=nz // 2, amp_source=1.0, omega_source=2.0e11, src_t0=15.0, src_tw=6.0, precision=precision)
    if not uniform:
        kw["dy"] = 1.25e-3
    boxes = [((nx // 3, ny // 3, nz // 3), (nx // 2, ny // 2 + 7, nz // 2 + 3), 4.0)]
    return cases.make(**kw), boxes


@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("uniform, n", [(True, (256, 128, 160)), (False, (90, 75, 101)), (True, (33, 200, 47))])
def test_sweep3_equals_two_sweep_large(engine, precision, uniform, n):
    p, boxes = _big3(precision, uniform, n)
    a, b = _pair(p, boxes)
    nx, ny, nz = n
    ijk = np.array([[nx // 2, ny // 2, nz // 2], [5, 6, 7], [nx - 2, ny - 2, nz - 2], [nx // 3, 1, nz - 1]],
                   dtype=np.int32)
    for s in (a, b):
        s.set_probes(ijk, 200)
        s.set_max_series(200)
    a.step(41)
    b.step(41)
    _same(a, b)
    a.step(30)
    b.step(30)
    _same(a, b)
    assert np.array_equal(a.probes(), b.probes())
    ta, va = a.max_series()
    tb, vb = b.max_series()
    assert np.array_equal(ta, tb) and np.array_equal(va, vb)
    assert a.max_e2() > 0


def test_sweep3_etotal_snapshot_and_checkpoint(engine, tmp_path):
    """|E|^2 snapshots from the 3-D sweep, and a checkpoint written at an odd step."""
    p, boxes = _big3(1, True, (90, 75, 101))
    a, b = _pair(p, boxes, dft=False)
    got = {}
    for s, key in ((a, "a"), (b, "b")):
        s.set_snapshots(7, 1 << 6, lambda t, c, arr, key=key: got.setdefault((key, t), np.array(arr)))
    a.step(29)
    b.step(29)
    a.sync()
    b.sync()
    for t in (0, 7, 14, 21, 28):
        assert np.array_equal(got[("a", t)], got[("b", t)]), t
    path = str(tmp_path / "odd3.h5")
    a.save(path)
    c = _sim(p, boxes, dft=False)
    c.load(path)
    for s in (a, b, c):
        s.step(12)
    _same(a, b)
    _same(c, b)


@pytest.mark.parametrize("precision", [1, 2])
def test_sweep3_handles_in_a_batch(engine, precision):
    """3-D single-sweep handles join a batch at odd and even steps and leave it again."""
    from luxum_gb300 import Batch

    specs = [_small("3d_pml_axis", precision), _small("3d_oblique", precision), _big3(precision, True, (90, 75, 101))]
    pairs = [_pair(p, boxes) for p, boxes in specs]
    for k, (a, b) in enumerate(pairs):
        a.step(3 + k)
        b.step(3 + k)
    batch = Batch(chunk=10)
    for a, _ in pairs:
        batch.add(a)
    batch.step(25)
    for _, b in pairs:
        b.step(25)
    for a, b in pairs:
        _same(a, b)
    batch.remove(pairs[2][0])
    for a, b in pairs:
        a.step(5)
        b.step(5)
        _same(a, b)


@pytest.mark.parametrize("precision", [1, 2])
def test_large_planar_member_steps_in_two_buffers(engine, precision):
    """A planar member of 2^21 cells or more takes the single-sweep kernel inside a batch, by
    value and in its two buffers, with its DFT plane read from the buffer of each step's
    parity; it must equal the same simulation on the two-sweep kernels stepped alone, across a
    join at an odd step, graph-captured chunks, an odd remainder and leaving again."""
    from luxum_gb300 import Batch

    kw = dict(isPlanar=1, Nx=1500, Ny=1, Nz=1460, **cases.pw((1, 0, 0), (0, 1, 0), ((30, 1469), (0, 0), (30, 1429))),
              **cases.pml(16), precision=precision)
    p = cases.make(**kw)
    boxes = [((600, 0, 500), (800, 1, 900), 3.0)]
    a, b = _pair(p, boxes)
    small, small_b = _pair(*_small("planar_pml_axis", precision))
    for s in (a, b):
        s.step(7)  # joins at an odd step
    batch = Batch(chunk=10)
    batch.add(a)
    batch.add(small)
    batch.step(43)  # four captured chunks and an odd remainder
    batch.step(20)
    b.step(63)
    small_b.step(63)
    _same(a, b)
    _same(small, small_b)
    batch.remove(a)
    a.step(5)
    b.step(5)
    _same(a, b)
    assert a.max_e2() > 0
