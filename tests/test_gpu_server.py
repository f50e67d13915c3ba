"""Serving (lx_server_*): continuous batching must not change any request's result.

Requests with different grids, step counts and arrival times share chunks; each must end
exactly where a handle stepped alone ends (fields, DFT flux, max|E|^2 bit for bit), while
the worker admits under the budget, cancels on request and fails only the request that
blows up.
"""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

W = 2 * np.pi * np.linspace(3e10, 1.5e11, 6)
REQS = [  # (case, steps, boxes, dft)
    ("planar_pml_axis", 137, [((20, 0, 20), (30, 1, 40), 4.0)], (0, 45, W, 1)),
    ("3d_pml_axis", 64, [((12, 10, 12), (18, 16, 20), 6.0)], (0, 20, W, 2)),
    ("planar_oblique", 250, [], (2, 28, W, 5)),
    ("3d_oblique", 40, [((10, 10, 10), (14, 20, 16), 2.5)], None),
]


def _params(name):
    p, _, _ = cases.build(name)
    p.precision = 1
    return p


def _solo(name, steps, boxes, dft):
    from luxum_gb300 import Sim

    s = Sim(_params(name))
    for lo, hi, eps in boxes:
        s.set_eps_box(lo, hi, eps)
    plane = None
    if dft is not None:
        axis, index, w, every = dft
        plane = s.add_dft_plane(axis, index, w, every=every)
    s.step(steps)
    return s, plane


def test_server_results_equal_solo(engine):
    from luxum_gb300 import Server

    with Server(chunk=50, tune_steps=5) as srv:
        ids = [srv.submit(_params(n), steps, boxes, dft) for n, steps, boxes, dft in REQS]
        for rid in ids:
            assert srv.wait(rid, 120.0) == "done", srv.error(rid)
        for rid, (n, steps, boxes, dft) in zip(ids, REQS):
            twin, plane = _solo(n, steps, boxes, dft)
            if dft is not None:
                assert np.array_equal(srv.flux(rid), twin.dft_flux(plane))
            assert srv.max_e2(rid) == twin.max_e2()
            t = srv.times(rid)
            assert 0 <= t[0] <= t[1] <= t[2]
            g = srv.take(rid, _params(n))
            assert g.t == steps
            for c in range(6):
                if np.prod(g.shape(c)):
                    assert np.array_equal(g.field(c), twin.field(c)), (n, c)
            g.close()
            twin.close()
        st = srv.stats()
        assert st["done"] == len(REQS) and st["running"] == 0 and st["queued"] == 0
        assert st["cell_updates"] > 0 and st["bytes_running"] == pytest.approx(0.0, abs=1.0)
        # every request's class was tuned on twins before it joined (all four are batched)
        table = srv.tune_table()
        classes = {(e["planar"], e["size_class"], e["slab_class"]) for e in table}
        assert len(classes) == len(table) == st["tuned_classes"] == 4
        assert all(e["march"] in (1, 2, 4, 8) and e["precision"] == 1 for e in table)
        assert st["tune_seconds"] > 0


def test_server_without_tuning_keeps_default_shapes(engine):
    from luxum_gb300 import Server

    n, steps, boxes, dft = REQS[0]
    with Server(chunk=50) as srv:  # no online tuning by default
        rid = srv.submit(_params(n), steps, boxes, dft)
        assert srv.wait(rid, 120.0) == "done", srv.error(rid)
        twin, plane = _solo(n, steps, boxes, dft)
        assert np.array_equal(srv.flux(rid), twin.dft_flux(plane))
        assert srv.tune_table() == [] and srv.stats()["tuned_classes"] == 0
        twin.close()


def test_server_with_a_preset_table(engine):
    """A table given at creation (say, from lx_batch_autotune on a sample of the expected
    requests) shapes the server's launches from the first chunk; results stay bit-identical."""
    from luxum_gb300 import Batch, Server, Sim

    sample = [Sim(_params(n)) for n, _, _, _ in REQS]
    b = Batch(chunk=10)
    for s in sample:
        b.add(s)
    b.autotune(3)
    table = b.tune_table()
    b.close()
    for s in sample:
        s.close()
    assert len(table) == 4
    table = [dict(e, march=(2, 4, 1, 8)[q]) for q, e in enumerate(table)]  # shapes other than the default
    with Server(chunk=50, tune_table=table) as srv:
        assert srv.tune_table() == table
        ids = [srv.submit(_params(n), steps, boxes, dft) for n, steps, boxes, dft in REQS]
        for rid in ids:
            assert srv.wait(rid, 120.0) == "done", srv.error(rid)
        for rid, (n, steps, boxes, dft) in zip(ids, REQS):
            twin, plane = _solo(n, steps, boxes, dft)
            if dft is not None:
                assert np.array_equal(srv.flux(rid), twin.dft_flux(plane))
            assert srv.max_e2(rid) == twin.max_e2()
            g = srv.take(rid, _params(n))
            for c in range(6):
                if np.prod(g.shape(c)):
                    assert np.array_equal(g.field(c), twin.field(c)), (n, c)
            g.close()
            twin.close()
        assert srv.stats()["tuned_classes"] == 0


def test_server_arrivals_while_others_run(engine):
    """Continuous batching: A and B are submitted first; C and D arrive once A is running and
    at least one chunk has finished, and join the batch between chunks while A and B are still
    on the GPU.  Every request must still equal its twin stepped alone, bit for bit (fields,
    flux and max|E|^2)."""
    import time

    from luxum_gb300 import Server

    first = [("3d_pml_axis", 3000, [((12, 10, 12), (18, 16, 20), 6.0)], (0, 20, W, 2)),
             ("planar_pml_axis", 2000, [((20, 0, 20), (30, 1, 40), 4.0)], (0, 45, W, 1))]
    late = [("planar_oblique", 150, [], (2, 28, W, 5)),
            ("3d_oblique", 90, [((10, 10, 10), (14, 20, 16), 2.5)], None)]
    with Server(chunk=20) as srv:
        ids = [srv.submit(_params(n), steps, boxes, dft) for n, steps, boxes, dft in first]
        t0 = time.monotonic()
        while not (srv.state(ids[0]) == "running" and srv.stats()["chunks"] >= 1):
            assert time.monotonic() - t0 < 60.0
            srv.wait(ids[0], 0.002)
        assert srv.state(ids[0]) == "running"  # A is mid-run when C and D arrive
        ids += [srv.submit(_params(n), steps, boxes, dft) for n, steps, boxes, dft in late]
        for rid in ids:
            assert srv.wait(rid, 120.0) == "done", srv.error(rid)
        ta = srv.times(ids[0])
        for rid in ids[2:]:
            tc = srv.times(rid)
            assert tc[0] > ta[1]  # submitted after A had started
        # at least one late request ran while A was still running
        assert min(srv.times(rid)[1] for rid in ids[2:]) < ta[2]
        for rid, (n, steps, boxes, dft) in zip(ids, first + late):
            twin, plane = _solo(n, steps, boxes, dft)
            if dft is not None:
                assert np.array_equal(srv.flux(rid), twin.dft_flux(plane)), n
            assert srv.max_e2(rid) == twin.max_e2(), n
            g = srv.take(rid, _params(n))
            assert g.t == steps
            for c in range(6):
                if np.prod(g.shape(c)):
                    assert np.array_equal(g.field(c), twin.field(c)), (n, c)
            g.close()
            twin.close()


def test_server_budget_and_cancel(engine):
    from luxum_gb300 import Server, device_bytes

    p = _params("planar_oblique")
    # room for one request at a time
    with Server(chunk=20, budget_bytes=1.5 * device_bytes(p)) as srv:
        a = srv.submit(p, 400)
        b = srv.submit(p, 400)
        c = srv.submit(p, 60)
        srv.cancel(b)  # still queued behind a
        assert srv.wait(b, 10.0) == "cancelled"
        assert srv.wait(c, 120.0) == "done"
        st = srv.stats()
        assert st["peak_running"] == 1
        assert st["cancelled"] == 1 and st["done"] == 2
        assert srv.times(a)[2] <= srv.times(c)[1]  # c started after a finished
        for rid in (a, b, c):
            srv.release(rid)
        # a running request leaves at the next chunk end
        d = srv.submit(p, 100000)
        while srv.state(d) != "running":
            srv.wait(d, 0.05)
        srv.cancel(d)
        assert srv.wait(d, 60.0) == "cancelled"


def test_server_fails_only_the_blown_up_request(engine):
    from luxum_gb300 import Server

    good = _params("planar_oblique")
    bad = _params("planar_oblique")
    bad.S = 3.0  # far past the Courant limit: FP32 overflows within ~50 steps
    with Server(chunk=25) as srv:
        rb = srv.submit(bad, 300)
        rg = srv.submit(good, 300)
        assert srv.wait(rb, 120.0) == "failed"
        assert "not finite" in srv.error(rb)
        assert srv.wait(rg, 120.0) == "done"
        twin, _ = _solo("planar_oblique", 300, [], None)
        g = srv.take(rg, good)
        assert np.array_equal(g.field(1), twin.field(1))


def test_server_rejects_bad_requests(engine):
    from luxum_gb300 import LuxumError, Server

    with Server() as srv:
        p = _params("planar_oblique")
        p.precision = 0
        with pytest.raises(LuxumError):
            srv.submit(p, 10)  # precision differs from the server's
        q = _params("planar_oblique")
        q.Nx = 2
        with pytest.raises(LuxumError):
            srv.submit(q, 10)  # reader::checkData-style rejection


def test_server_material_arrays(engine):
    """Requests carrying material arrays (the batch workload's lens maps) equal solo runs."""
    from luxum_gb300 import Server, Sim, field_shape

    rng = np.random.default_rng(9)
    planar, three = _params("planar_pml_axis"), _params("3d_pml_axis")
    Fp = {1: (rng.random(field_shape(planar, 1)) < 0.3) * 1.5}
    F3 = {c: (rng.random(field_shape(three, c)) < 0.2) * 3e-6 for c in range(3)}
    with Server(chunk=20) as srv:
        a = srv.submit(planar, 90, material=Fp, material_scale=1.0)
        b = srv.submit(three, 50, boxes=[((12, 10, 12), (18, 16, 20), 6.0)], material=F3, material_scale=1e6)
        assert srv.wait(a, 120.0) == "done" and srv.wait(b, 120.0) == "done"
        ga, gb = srv.take(a, planar), srv.take(b, three)
    sa, sb = Sim(planar), Sim(three)
    sa.set_material(1, Fp[1], 1.0)
    for c in range(3):
        sb.set_material(c, F3[c], 1e6)
    sb.set_eps_box((12, 10, 12), (18, 16, 20), 6.0)
    sa.step(90)
    sb.step(50)
    for g, s in ((ga, sa), (gb, sb)):
        for c in range(6):
            if np.prod(s.shape(c)):
                assert np.array_equal(g.field(c), s.field(c)), c


def test_server_destroy_with_work_in_flight(engine):
    """Destroying a server cancels what is queued and running and frees every handle."""
    from luxum_gb300 import Server

    p = _params("planar_oblique")
    srv = Server(chunk=10, max_running=1)
    ids = [srv.submit(p, 100000) for _ in range(3)]
    while srv.state(ids[0]) != "running":
        srv.wait(ids[0], 0.05)
    srv.close()  # returns after the chunk in flight
    # a fresh server on the same device still works
    with Server(chunk=10) as again:
        rid = again.submit(p, 30)
        assert again.wait(rid, 60.0) == "done"


def test_fp16_storage_requests(engine):
    """A server of FP16-storage requests equals the same simulations stepped alone."""
    from luxum_gb300 import Server, Sim

    p = _params("3d_pml_axis")
    p.precision = 2
    with Server(precision=2, chunk=16) as srv:
        rid = srv.submit(p, 40, [((12, 10, 12), (18, 16, 20), 6.0)])
        assert srv.wait(rid, 60.0) == "done"
        g = srv.take(rid, p)
    s = Sim(p)
    s.set_eps_box((12, 10, 12), (18, 16, 20), 6.0)
    s.step(40)
    for c in range(6):
        assert np.array_equal(g.field(c), s.field(c)), c


def test_trim_device_memory_after_teardown(engine):
    """Destroyed handles give their memory back to the device pool; lx_trim_device_memory
    returns it to the driver, and later handles allocate and step as before."""
    from luxum_gb300 import Sim, trim_device_memory

    n, steps, boxes, dft = REQS[1]
    for s in [Sim(_params(n)) for _ in range(4)]:
        s.step(3)
        s.close()
    trim_device_memory()
    twin, _ = _solo(n, steps, boxes, dft)
    again, _ = _solo(n, steps, boxes, dft)
    for c in range(6):
        if np.prod(again.shape(c)):
            assert np.array_equal(again.field(c), twin.field(c))
    twin.close()
    again.close()


def test_server_config_validation(engine):
    """A table count without a table, and negative tuning steps, are refused at creation."""
    import ctypes as C

    from luxum_gb300 import _ffi

    lib = _ffi.lib()
    for field, value in (("tune_entries", 2), ("tune_steps", -1)):
        cfg = _ffi.ServerConfig()
        lib.lx_server_config_init(C.byref(cfg))
        setattr(cfg, field, value)
        h = C.c_void_p()
        assert lib.lx_server_create(C.byref(cfg), C.byref(h)) == 1  # LX_ERR_INVALID
        assert not h.value
