"""Parity at the benchmark configurations' full grid sizes.

- The 2-D CPML configuration (512 x 512, 2000 steps, TF/SF box [30,481]^2, eps_r 10.89
  block [224,288)^2, 20-cell CPML with kappa 5 and a_max 0.05): the whole run against the
  oracle, which finishes it in seconds.
- The 3-D drop-in workload (256^3, CPML 16, TF/SF box [32,223]^3, eps_r 6 cube from the
  material formula, max|E|^2 every step): 300 of its 1000 steps against the oracle (the
  wave has crossed the cube), then properties that hold at any length: a run is
  deterministic, and checkpoint + resume continues bit for bit.

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


def test_3d_dropin_workload_full_grid(engine, tmp_path):
    sys.path.insert(0, ROOT)
    import bench
    from luxum_gb300 import Sim
    from oracle.oracle import OracleSim

    p = bench.workload_params(0)
    g, o = Sim(p), OracleSim(p, threads=os.cpu_count() or 1)
    for c in range(3):
        F = bench.material(o.shape(c))
        g.set_material(c, F, 1e6)
        o.set_material(c, F, 1e6)
    g.step(300)
    o.step(300)
    for c, err in _errors(g, o).items():
        assert err <= TOL, (c, err)
    assert g.max_e2() == pytest.approx(o.max_e2(), rel=TOL)
    o.close()
    # any-length properties on the same grid
    g.save(tmp_path / "ck.h5")
    g.step(200)
    h = Sim(p)
    for c in range(3):
        h.set_material(c, bench.material(h.shape(c)), 1e6)
    h.load(tmp_path / "ck.h5")
    h.step(200)
    twin = Sim(p)
    for c in range(3):
        twin.set_material(c, bench.material(twin.shape(c)), 1e6)
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
