"""Batched stepping (lx_batch_*): every member must evolve exactly as it does alone.

Members of mixed kinds (planar and 3-D, uniform and non-uniform spacing, with and without
CPML, TF/SF and DFT planes) share launches; their fields, DFT accumulators and max|E|^2
must equal those of twin handles stepped one by one, bit for bit, across graph replays,
steps taken alone in between and removal of a member.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

NAMES = ["planar_pml_axis", "planar_oblique", "3d_pml_axis", "3d_pml_pulse_nonuniform"]


def _make(name, precision):
    from luxum_gb300 import Sim

    p, steps, boxes = cases.build(name)
    p.precision = precision
    s = Sim(p)
    for lo, hi, eps in boxes:
        s.set_eps_box(lo, hi, eps)
    if name in ("planar_pml_axis", "3d_pml_axis"):
        w = 2 * np.pi * np.linspace(3e10, 1.5e11, 5)
        s.add_dft_plane(0, 20, w, every=2 if name == "3d_pml_axis" else 1)
    return s


def _same(a, b):
    for c in range(6):
        if np.prod(a.shape(c)) == 0:
            continue
        assert np.array_equal(a.field(c), b.field(c)), c
    for plane in getattr(a, "_dft", {}):
        assert np.array_equal(a.dft(plane), b.dft(plane))
    assert a.max_e2() == b.max_e2()
    assert a.t == b.t


@pytest.mark.parametrize("precision", [1, 0, 2])
def test_batch_equals_solo(engine, precision):
    from luxum_gb300 import Batch

    members = [_make(n, precision) for n in NAMES]
    twins = [_make(n, precision) for n in NAMES]
    batch = Batch(chunk=10)
    for m in members:
        batch.add(m)
    assert len(batch) == 4
    batch.step(37)  # 3 graph replays + 7 direct steps
    for t in twins:
        t.step(37)
    for m, t in zip(members, twins):
        _same(m, t)
    members[2].step(5)  # a member steps alone between batch steps
    twins[2].step(5)
    batch.step(13)
    for t in twins:
        t.step(13)
    for m, t in zip(members, twins):
        _same(m, t)
    batch.remove(members[1])
    batch.step(20)
    for i in (0, 2, 3):
        twins[i].step(20)
    for i in (0, 2, 3):
        _same(members[i], twins[i])
    batch.close()


def test_batch_rejects_mixed_precision(engine):
    from luxum_gb300 import Batch, LuxumError

    a, b = _make("planar_oblique", 1), _make("planar_oblique", 0)
    batch = Batch()
    batch.add(a)
    with pytest.raises(LuxumError):
        batch.add(b)


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_device_bytes_estimate(engine, name):
    """lx_params_device_bytes (host-only) agrees with what a created handle holds."""
    from luxum_gb300 import Sim, device_bytes

    p, steps, boxes = cases.build(name)
    est = device_bytes(p)
    s = Sim(p)
    held = s.info()["device_bytes"]
    assert 0.9 * held <= est <= 1.1 * held + 4096, (est, held)
    s.close()


def test_batch_async_equals_blocking(engine):
    """lx_batch_step_async + lx_batch_wait give what lx_batch_step gives, and host work
    between the two (creating a handle, stepping it alone) does not disturb the chunk."""
    from luxum_gb300 import Batch

    a = [_make(n, 1) for n in NAMES]
    b = [_make(n, 1) for n in NAMES]
    ba, bb = Batch(chunk=10), Batch(chunk=10)
    for m in a:
        ba.add(m)
    for m in b:
        bb.add(m)
    for _ in range(3):
        ba.step_async(20)
        extra = _make("planar_oblique", 1)
        extra.step(3)
        extra.close()
        ba.wait()
        bb.step(20)
    for m, t in zip(a, b):
        _same(m, t)
    ba.close()
    bb.close()


@pytest.mark.parametrize("march", [1, 2, 8])
def test_batch_tile_shape_does_not_change_results(engine, march):
    from luxum_gb300 import Batch

    members = [_make(n, 1) for n in NAMES]
    twins = [_make(n, 1) for n in NAMES]
    batch = Batch(chunk=10)
    batch.set_march(march, march)
    for m in members:
        batch.add(m)
    batch.step(37)
    for t in twins:
        t.step(37)
    for m, t in zip(members, twins):
        _same(m, t)
    batch.close()


def _class_members(precision):
    """Members spanning every tuned axis: planar and 3-D, size classes 5 to 8, x slab classes
    0 (no CPML), 1 (up to 8 cells), 2 (up to 16) and 3 (deeper), uniform and non-uniform."""
    from luxum_gb300 import Sim

    extra = {
        "planar_pml12": dict(isPlanar=1, Nx=96, Ny=1, Nz=96, **cases.pw((1, 0, 0), (0, 1, 0), ((18, 77), (0, 0), (18, 77))),
                             **cases.pml(12)),
        "3d_pml20": dict(isPlanar=0, Nx=60, Ny=58, Nz=62, **cases.pw((1, 0, 0), (0, 0, 1), ((24, 35), (23, 34), (24, 37))),
                         **cases.pml(20, kappa=15, a_max=0.0)),
    }
    out = [_make(n, precision) for n in ("planar_pml_axis", "planar_oblique", "3d_pml_axis", "3d_oblique",
                                         "3d_pml_pulse_nonuniform")]
    for kw in extra.values():
        p = cases.make(**kw)
        p.precision = precision
        out.append(Sim(p))
    return out


@pytest.mark.parametrize("precision", [1, 0, 2])
def test_tune_table_classes_do_not_change_results(engine, precision):
    """Every class of member takes its own march from the table (1, 2, 4, 8 in turn), so
    members of one launch group split by march; results stay bit-identical to solo steps."""
    from luxum_gb300 import Batch

    members = _class_members(precision)
    twins = _class_members(precision)
    classes = []
    for m in members:
        k = m.tune_class()
        if k not in classes:
            classes.append(k)
    assert {k["slab_class"] for k in classes} == {0, 1, 2, 3}
    assert {k["planar"] for k in classes} == {0, 1}
    assert len({k["size_class"] for k in classes}) >= 3
    assert all(k["precision"] == precision for k in classes)
    table = [dict(k, march=(1, 2, 4, 8)[q % 4]) for q, k in enumerate(classes)]
    batch = Batch(chunk=10)
    batch.set_tune_table(table)
    assert batch.tune_table() == table
    for m in members:
        batch.add(m)
    batch.step(37)
    for t in twins:
        t.step(37)
    for m, t in zip(members, twins):
        _same(m, t)
    # the tuner records one entry per class and leaves the members' results unchanged
    batch.set_tune_table([])
    batch.autotune(3)
    got = batch.tune_table()
    assert sorted((e["planar"], e["size_class"], e["slab_class"]) for e in got) == \
        sorted((k["planar"], k["size_class"], k["slab_class"]) for k in classes)
    assert all(e["march"] in (1, 2, 4, 8) for e in got)
    batch.step(11)
    for t in twins:
        t.step(11)
    for m, t in zip(members, twins):
        _same(m, t)
    batch.close()


def test_tune_table_validation_and_member_tuning(engine):
    from luxum_gb300 import Batch, LuxumError

    batch = Batch(chunk=10)
    k = dict(planar=1, size_class=6, precision=1, slab_class=1)
    with pytest.raises(LuxumError):
        batch.set_tune_table([dict(k, march=3)])
    with pytest.raises(LuxumError):
        batch.set_tune_table([dict(k, slab_class=4, march=2)])
    batch.set_tune_table([dict(k, march=2), dict(k, march=4)])  # the last entry of a class wins
    assert batch.tune_table() == [dict(k, march=4)]
    s = _make("planar_pml_axis", 1)
    assert s.tune_class() == k
    m = batch.tune_member(s, 3)
    assert m in (1, 2, 4, 8)
    assert batch.tune_table() == [dict(k, march=m)]
    assert s.t == 0  # the handle itself is not stepped
    batch.close()


def test_tune_table_errors(engine):
    """Tuning a handle of another precision than the batch's members is refused; an empty
    table clears the batch's picks; a batch without batched members tunes nothing."""
    from luxum_gb300 import Batch, LuxumError

    batch = Batch(chunk=10)
    m = _make("planar_pml_axis", 1)
    batch.add(m)
    s64 = _make("planar_pml_axis", 0)
    with pytest.raises(LuxumError):
        batch.tune_member(s64, 3)
    k = m.tune_class()
    batch.set_tune_table([dict(k, march=2)])
    assert batch.tune_table() == [dict(k, march=2)]
    batch.set_tune_table([])
    assert batch.tune_table() == []
    batch.remove(m)
    assert batch.autotune(3) == batch.march()  # nothing to time: the per-dimension march stays
    assert batch.tune_table() == []
    batch.close()


def test_batch_autotune_leaves_members_untouched(engine):
    from luxum_gb300 import Batch

    members = [_make(n, 1) for n in NAMES]
    twins = [_make(n, 1) for n in NAMES]
    batch = Batch(chunk=10)
    for m in members:
        batch.add(m)
    batch.step(13)
    before = [[m.field(c) if np.prod(m.shape(c)) else None for c in range(6)] for m in members]
    got = batch.autotune(10)
    assert got[0] in (1, 2, 4, 8) and got[1] in (1, 2, 4, 8)
    assert batch.march() == got
    for m, f in zip(members, before):
        assert m.t == 13
        for c in range(6):
            if f[c] is not None:
                assert np.array_equal(m.field(c), f[c])
    batch.step(24)
    for t in twins:
        t.step(37)
    for m, t in zip(members, twins):
        _same(m, t)
    batch.close()


def test_member_changes_after_joining(engine):
    """A DFT plane added to a member after it joined is sampled from the next batch step;
    outputs a batch cannot serve (probes, snapshots) are refused while the handle is a member."""
    from luxum_gb300 import Batch, LuxumError

    m, t = _make("planar_oblique", 1), _make("planar_oblique", 1)
    batch = Batch(chunk=10)
    batch.add(m)
    batch.step(10)
    t.step(10)
    w = 2 * np.pi * np.linspace(3e10, 1.5e11, 5)
    pm = m.add_dft_plane(2, 25, w, every=2)
    pt = t.add_dft_plane(2, 25, w, every=2)
    batch.step(25)
    t.step(25)
    assert np.array_equal(m.dft(pm), t.dft(pt))
    _same(m, t)
    with pytest.raises(LuxumError):
        m.set_probes([[10, 0, 10]], capacity=5)
    with pytest.raises(LuxumError):
        m.set_snapshots(5, 1 << 1, lambda *a: None)
    batch.close()


def _cube(n, precision, pulse=False):
    from luxum_gb300 import Sim

    kw = dict(isPlanar=0, Nx=n + 2, Ny=n, Nz=n, precision=precision,
              **cases.pw((1, 0, 0), (0, 0, 1), ((12, n - 11), (11, n - 12), (11, n - 12))), **cases.pml(8, kappa=15))
    if pulse:
        kw.update(usePS=1, source_kind=1, Nx_source=n // 2, Ny_source=n // 2, Nz_source=n // 3, amp_source=1.0,
                  omega_source=2.0e11, src_t0=12.0, src_tw=5.0)
    s = Sim(cases.make(**kw))
    s.set_eps_box((n // 3, n // 3, n // 3), (n // 2, n // 2, n // 2), 5.0)
    s.add_dft_plane(0, n // 2, 2 * np.pi * np.linspace(3e10, 1.5e11, 4), every=2)
    return s


@pytest.mark.parametrize("precision", [1, 0])
def test_large_3d_members_launched_one_by_one(engine, precision):
    """3-D members of 2^18 cells or more take one kernel pair each on four streams; with a
    small 3-D member (the batched kernel) and a planar one, all equal their solo twins."""
    from luxum_gb300 import Batch

    def make():
        return [_cube(64, precision), _cube(66, precision, pulse=True), _cube(70, precision), _cube(72, precision),
                _cube(80, precision, pulse=True), _make("3d_pml_axis", precision), _make("planar_pml_axis", precision)]

    members, twins = make(), make()
    assert members[0].info()["cells"] >= 1 << 18 and members[5].info()["cells"] < 1 << 18
    batch = Batch(chunk=10)
    for m in members:
        batch.add(m)
    batch.step(25)  # graph replays and direct steps
    for t in twins:
        t.step(25)
    for m, t in zip(members, twins):
        _same(m, t)
    members[1].step(3)  # a member steps alone between batch steps
    twins[1].step(3)
    batch.step(10)
    for t in twins:
        t.step(10)
    for m, t in zip(members, twins):
        _same(m, t)
