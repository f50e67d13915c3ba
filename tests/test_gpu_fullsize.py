"""Parity at the benchmark configurations' full grid sizes.

- The 2-D CPML configuration (512 x 512, 2000 steps, TF/SF box [30,481]^2, eps_r 10.89
  block [224,288)^2, 20-cell CPML with kappa 5 and a_max 0.05): the whole run against the
  oracle, which finishes it in seconds.
- The 3-D drop-in workload (256^3, CPML 16, TF/SF box [32,223]^3, eps_r 6 cube from the
  material formula, max|E|^2 every step): all 1000 steps against the oracle, with its four
  Ex..Hz snapshots and its 8-probe series; then properties that hold at any length: a run
  is deterministic, and checkpoint + resume continues bit for bit.

Tolerance: relative L2 <= 1e-12 per component against its field group's norm (FP64).
"""
import os
import sys

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL = 1e-12
OWN_TOL = 1e-9  # own-norm figure of components above 1e-6 of their group


def _errors(g, o):
    shapes = {c: o.shape(c) for c in range(6)}
    return cases.field_errors(g.field, o.field, shapes)


def test_2d_cpml_config_full_run(engine):
    from luxum_gb300 import Sim
    from oracle.oracle import OracleSim

    p = cases.make(isPlanar=1, Nx=512, Ny=1, Nz=512, num_timesteps=2000,
                   **cases.pw((1, 0, 0), (0, 1, 0), ((30, 481), (0, 0), (30, 481)), off=26.0),
                   **cases.pml(20, kappa=5.0, a_max=0.05))
    g, o = Sim(p), OracleSim(p, threads=os.cpu_count() or 1)
    for s in (g, o):
        s.set_eps_box((224, 0, 224), (288, 1, 288), 10.89)
    g.step(2000)
    o.step(2000)
    for c, err in _errors(g, o).items():
        assert err <= TOL, (c, err)
    assert g.max_e2() == pytest.approx(o.max_e2(), rel=TOL)


def test_3d_dropin_workload_full_run(engine):
    """The whole drop-in workload, all 1000 steps, as the bench runs it: Ex..Hz snapshots at
    t = 0, 250, 500, 750 (taken after the E update of step t, three_dim_pml.cc:279's
    cadence semantics), the 8 seeded probes' six components every step, the final fields and
    max|E|^2, each against the oracle.  Snapshots and final fields: group-normalised and
    own-norm relative L2 (own-norm where the component is more than 1e-6 of its group);
    probe series: relative L2 of each probe component's 1000-step series against the largest
    series of its field group."""
    sys.path.insert(0, ROOT)
    import bench
    from luxum_gb300 import Sim
    from oracle.oracle import OracleSim

    p = bench.workload_params(0)
    g = Sim(p)
    for c in range(3):
        g.set_material(c, bench.material(g.shape(c)), 1e6)
    ijk = bench.probe_points()
    g.set_probes(ijk, bench.STEPS)
    snaps = {}

    def keep(t, comp, arr):
        snaps[(t, comp)] = np.array(arr, copy=True)

    g.set_snapshots(bench.SNAP_EVERY, 0x3F, keep)
    g.step(bench.STEPS)
    g.sync()
    gp = g.probes()
    assert sorted({t for t, _ in snaps}) == [0, 250, 500, 750] and len(snaps) == 24

    o = OracleSim(p, threads=os.cpu_count() or 1)
    for c in range(3):
        o.set_material(c, bench.material(o.shape(c)), 1e6)
    o.set_probes(ijk, bench.STEPS)
    shapes = {c: o.shape(c) for c in range(6)}
    report = {}
    done = 0
    for t in (0, 250, 500, 750):
        o.step(t + 1 - done)  # after step t
        done = t + 1
        report[t] = _both_errors(lambda c: snaps[(t, c)], o.field, shapes)
    o.step(bench.STEPS - done)
    report["final"] = _both_errors(g.field, o.field, shapes)
    assert g.max_e2() == pytest.approx(o.max_e2(), rel=TOL)
    op = o.probes()
    assert gp.shape == op.shape == (bench.STEPS, 8, 6)
    perr = 0.0
    for grp in ((0, 1, 2), (3, 4, 5)):
        scale = max(float(np.linalg.norm(op[:, q, c])) for q in range(8) for c in grp)
        for q in range(8):
            for c in grp:
                perr = max(perr, float(np.linalg.norm(gp[:, q, c] - op[:, q, c])) / scale)
    print("256^3 FP64 1000 steps vs oracle:", report, "probe series worst", perr)
    for key, (grp, own) in report.items():
        for c, e in grp.items():
            assert e <= TOL, (key, "group-normalised", c, e)
        for c, e in own.items():
            assert e <= OWN_TOL, (key, "own-norm", c, e)
    assert perr <= TOL
    o.close()
    g.close()


def _both_errors(get_a, get_b, shapes):
    grp = cases.field_errors(get_a, get_b, shapes)
    own = {}
    for group in ((0, 1, 2), (3, 4, 5)):
        bs = {c: get_b(c) for c in group}
        gn = float(np.sqrt(sum(np.linalg.norm(b) ** 2 for b in bs.values())))
        for c in group:
            nb = float(np.linalg.norm(bs[c]))
            if nb > 1e-6 * gn:
                own[c] = float(np.linalg.norm(get_a(c) - bs[c])) / nb
    return grp, own


def test_3d_dropin_checkpoint_and_determinism(engine, tmp_path):
    """Any-length properties on the full 256^3 grid: a run is deterministic, and checkpoint +
    resume continues bit for bit."""
    sys.path.insert(0, ROOT)
    import bench
    from luxum_gb300 import Sim

    p = bench.workload_params(0)

    def fresh():
        s = Sim(p)
        for c in range(3):
            s.set_material(c, bench.material(s.shape(c)), 1e6)
        return s

    g = fresh()
    g.step(300)
    g.save(tmp_path / "ck.h5")
    g.step(200)
    h = fresh()
    h.load(tmp_path / "ck.h5")
    h.step(200)
    twin = fresh()
    twin.step(500)
    for c in range(6):
        a = g.field(c)
        assert np.array_equal(a, h.field(c)), c      # resumed run
        assert np.array_equal(a, twin.field(c)), c   # deterministic


def test_full_grid_linearity(engine):
    """256^3 with CPML and a dielectric cube, 1000 steps, hard CW point source: doubling the
    source amplitude doubles every field exactly (every operation is linear and x2 is exact
    in binary floating point while no value is subnormal, which holds in FP64 here; FP32's
    light-cone edge reaches subnormals).  A property of the whole update at the workload's
    full size and length, independent of the oracle."""
    precision = 0
    sys.path.insert(0, ROOT)
    import bench
    from luxum_gb300 import Sim

    fields = []
    for amp in (1.0, 2.0):
        p = bench.workload_params(precision)
        p.usePW = 0
        p.usePS, p.Nx_source, p.Ny_source, p.Nz_source = 1, 128, 128, 100
        p.amp_source, p.omega_source = amp, 2.0e9  # both kept as int by the reference
        s = Sim(p)
        for c in range(3):
            s.set_material(c, bench.material(s.shape(c)), 1e6)
        s.step(1000)
        fields.append([s.field(c) for c in range(6)])
        s.close()
    for c in range(6):
        assert np.array_equal(fields[1][c], 2.0 * fields[0][c]), c
        assert np.abs(fields[0][c]).max() > 0
