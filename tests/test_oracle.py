"""The oracle on the CPU: golden fixtures, physics properties, determinism.

The reference has no tests and cannot be built here, so the oracle is pinned by
(a) its committed golden outputs (regenerated only by tests/golden/make_golden.py),
(b) physical properties of the reference algorithm it restates: a TF/SF plane wave is a
    clean Gaussian inside the total-field box and leaves almost nothing outside it; the
    planar drivers inject with the opposite sign (maxwell.cc:206 vs :289); a PEC cavity
    without sources keeps a bounded field; the CPML profiles have the graded shape of
    maxwell.cc:997-1280,
(c) OpenMP thread-count invariance (every loop writes disjoint cells).
"""
import json
import pathlib

import numpy as np
import pytest

import cases
from cases import rel_l2

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
MANIFEST = json.loads((GOLDEN / "manifest.json").read_text())


def _run(name, threads=2, steps=None):
    from oracle.oracle import OracleSim

    p, n, boxes = cases.build(name)
    o = OracleSim(p, threads=threads)
    for lo, hi, eps in boxes:
        o.set_eps_box(lo, hi, eps)
    return o, p, (n if steps is None else steps)


def _probe_points(p):
    rng = np.random.default_rng(2026)
    return np.stack([rng.integers(0, n, 8) for n in (p.Nx, p.Ny if not p.isPlanar else 1, p.Nz)], axis=1)


@pytest.mark.parametrize("name", sorted(MANIFEST["cases"]))
def test_golden(name):
    o, p, steps = _run(name, threads=3)
    g = np.load(GOLDEN / f"{name}.npz")
    o.set_probes(_probe_points(p), steps)
    o.step(steps)
    assert np.array_equal(g["probe_ijk"], _probe_points(p))
    assert rel_l2(o.probes(), g["probes"]) <= 1e-13
    assert abs(o.max_e2() - float(g["max_e2"])) <= 1e-13 * abs(float(g["max_e2"]))
    for c in range(6):
        if f"f{c}" not in g:
            continue
        f = o.field(c)
        sub = f if p.isPlanar else f[::3, ::3, ::3]
        assert rel_l2(sub, g[f"f{c}"]) <= 1e-13, c
        assert abs(np.linalg.norm(f) - float(g[f"norm{c}"])) <= 1e-13 * float(g[f"norm{c}"])


def test_thread_count_invariance():
    a, p, n = _run("3d_pml_axis", threads=1, steps=25)
    b, _, _ = _run("3d_pml_axis", threads=7, steps=25)
    a.step(25)
    b.step(25)
    for c in range(6):
        assert np.array_equal(a.field(c), b.field(c))


def test_tfsf_pulse_is_clean_and_contained():
    from oracle.oracle import OracleSim

    p = cases.make(isPlanar=0, Nx=64, Ny=64, Nz=64, **cases.pw((1, 0, 0), (0, 0, 1), ((12, 51), (12, 51), (12, 51))))
    o = OracleSim(p, threads=4)
    o.step(130)
    ex, ey, ez = o.field(0), o.field(1), o.field(2)
    assert abs(ez).max() > 0.99                      # unit-amplitude pulse inside the box
    assert abs(ex).max() < 2e-3 and abs(ey).max() < 2e-3   # polarisation kept
    assert abs(ez[:, :10]).max() < 2e-3              # scattered-field zone stays quiet
    assert abs(ez[:10]).max() < 2e-3
    # the Gaussian of maxwell.cc:71 (sigma = 2e-4 m^2) centred at x = 0.5 t - off_pw cells
    x = np.arange(64) * 1e-3
    centre = (0.5 * 129 - 30.0) * 1e-3  # E at step t=129 is driven by the H-curl term at time t (maxwell.cc:397)
    prof = ez[14:50, 32, 32]
    ref = np.exp(-((x[14:50] - centre) ** 2) / (pow(10, -4) / 0.5))
    assert np.max(np.abs(prof - ref)) < 0.05


def test_planar_wave_has_opposite_sign():
    from oracle.oracle import OracleSim

    p = cases.make(isPlanar=1, Nx=96, Ny=1, Nz=96, **cases.pw((1, 0, 0), (0, 1, 0), ((12, 83), (0, 0), (12, 83))))
    o = OracleSim(p, threads=2)
    o.step(150)
    ey = o.field(1)[:, 0, :]
    assert ey.min() < -0.99 and ey.max() < 0.01
    assert abs(ey[:, :10]).max() < 2e-3


def test_pec_cavity_stays_bounded():
    from oracle.oracle import OracleSim

    p = cases.make(isPlanar=0, Nx=20, Ny=18, Nz=22)
    o = OracleSim(p, threads=2)
    rng = np.random.default_rng(3)
    e = rng.standard_normal(o.shape(2))
    e[0] = e[-1] = 0
    e[:, 0] = e[:, -1] = 0
    o.set_field(2, e)
    e0 = np.linalg.norm(e)
    for _ in range(10):
        o.step(40)
        tot = sum(np.linalg.norm(o.field(c)) ** 2 for c in range(3)) ** 0.5
        assert tot < 3 * e0


def test_cpml_profiles_shape():
    from oracle.oracle import OracleSim

    p, _, _ = cases.build("planar_pml_axis")  # 8-cell layer, kappa 5, a_max 0.05
    o = OracleSim(p)
    n = p.Nx
    sig = o.profile(0, 0, True, n)
    kap = o.profile(1, 0, True, n)
    a = o.profile(2, 0, True, n)
    b = o.profile(3, 0, True, n)
    c = o.profile(4, 0, True, n)
    d = 8.0
    assert sig[0] > sig[3] > 0 and np.all(sig[8:n - 8] == 0) and sig[n - 1] > 0
    assert kap[0] == pytest.approx(5.0) and np.all(kap[8:n - 8] == 1)
    assert a[int(d - 1)] == pytest.approx(0.05) and a[0] == 0
    assert np.all(c[sig == 0] == 0) and np.all(b[8:n - 8] == 1)
    # the reference subtracts a in b = exp(-(sigma/kappa - a)/eps0*dt) (maxwell.cc:1215): b > 1 near the inner edge
    assert b[6] > 1.0
    h = o.profile(0, 0, False, n - 1)
    assert h.shape == (n - 1,) and h[0] > 0


def test_invalid_rejected():
    from oracle.oracle import OracleError, OracleSim

    with pytest.raises(OracleError):
        OracleSim(cases.make(isPlanar=1, Nx=30, Ny=1, Nz=30, usePS=1, Nx_source=4, Nz_source=4))
