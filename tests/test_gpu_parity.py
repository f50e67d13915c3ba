"""FP64 parity of the CUDA engine against the oracle (the reference's drivers restated).

Tolerance: relative L2 <= 1e-12 per field component, relative to the norm of its field
group (||E|| or ||H||, see cases.field_errors), FP64.  The kernels differ from the reference
only by FMA contraction, reciprocal multiplies and exp() last-bit rounding.
"""
import numpy as np
import pytest

import cases
from cases import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _pair(name, engine):
    from luxum_gb300 import Sim
    from oracle.oracle import OracleSim

    p, steps, boxes = cases.build(name)
    g = Sim(p)
    o = OracleSim(p, threads=4)
    for lo, hi, eps in boxes:
        g.set_eps_box(lo, hi, eps)
        o.set_eps_box(lo, hi, eps)
    return g, o, steps


def _compare(g, o, tag):
    shapes = {c: o.shape(c) for c in range(6)}
    for c in range(6):
        assert g.shape(c) == shapes[c], (tag, c)
    errs = cases.field_errors(g.field, o.field, shapes)
    for c, err in errs.items():
        assert err <= TOL, f"{tag}: component {c} rel-L2 {err:.3e}"
    m_g, m_o = g.max_e2(), o.max_e2()
    assert abs(m_g - m_o) <= TOL * max(abs(m_o), 1e-300), f"{tag}: max|E|^2 {m_g!r} vs {m_o!r}"


@pytest.mark.parametrize("name", sorted(cases.CASES))
def test_fp64_matches_oracle(name, engine):
    g, o, steps = _pair(name, engine)
    half = steps // 2
    g.step(half)
    o.step(half)
    _compare(g, o, f"{name} t={half}")
    g.step(steps - half)
    o.step(steps - half)
    _compare(g, o, f"{name} t={steps}")
    # the fields are not trivially zero
    assert max(float(np.abs(o.field(c)).max()) for c in range(6) if np.prod(o.shape(c)) > 0) > 1e-6
    g.close()


def test_material_formula_matches(engine):
    """Cb = dt/(eps0*(1+F*1e6)) from a material array (three_dim_pml.cc:109-128)."""
    from luxum_gb300 import Sim
    from oracle.oracle import OracleSim

    p, steps, _ = cases.build("3d_pml_axis")
    g, o = Sim(p), OracleSim(p, threads=4)
    rng = np.random.default_rng(7)
    for c in range(3):
        F = (rng.random(o.shape(c)) < 0.2) * 5e-6 * rng.random(o.shape(c))
        g.set_material(c, F, 1e6)
        o.set_material(c, F, 1e6)
    g.step(40)
    o.step(40)
    _compare(g, o, "material")


def test_dft_plane_matches(engine):
    """FP64 running-DFT planes: accumulators and flux against the oracle."""
    from luxum_gb300 import Sim
    from oracle.oracle import OracleSim

    p, steps, boxes = cases.build("3d_pml_axis")
    g, o = Sim(p), OracleSim(p, threads=4)
    for lo, hi, eps in boxes:
        g.set_eps_box(lo, hi, eps)
        o.set_eps_box(lo, hi, eps)
    w = 2 * np.pi * np.linspace(2e10, 1.2e11, 7)
    ids = [(g.add_dft_plane(0, 11, w), o.add_dft_plane(0, 11, w)), (g.add_dft_plane(2, 20, w, every=2),
                                                                    o.add_dft_plane(2, 20, w, every=2))]
    g.step(steps)
    o.step(steps)
    for gi, oi in ids:
        a, b = g.dft(gi), o.dft(oi)
        assert a.shape == b.shape
        assert np.linalg.norm(a - b) <= 1e-11 * np.linalg.norm(b)
    # flux: Re(E_y conj(H_z) - E_z conj(H_y)) summed over the x-plane, times dy*dz
    b = o.dft(ids[0][1])
    ref = (np.real(b[:, 0] * np.conj(b[:, 3]) - b[:, 1] * np.conj(b[:, 2])).sum(axis=(1, 2))) * p.dy * p.dz
    assert np.allclose(g.dft_flux(ids[0][0]), ref, rtol=1e-9, atol=1e-9 * np.abs(ref).max())


def test_probes_match(engine):
    from luxum_gb300 import Sim
    from oracle.oracle import OracleSim

    p, steps, boxes = cases.build("3d_pml_axis")
    g, o = Sim(p), OracleSim(p, threads=4)
    rng = np.random.default_rng(2026)
    ijk = np.stack([rng.integers(0, n, 8) for n in (p.Nx, p.Ny, p.Nz)], axis=1)
    ijk[0] = (p.Nx - 1, p.Ny - 1, p.Nz - 1)  # outside several extents -> zeros
    g.set_probes(ijk, 100)
    o.set_probes(ijk, 100)
    g.step(30)
    o.step(30)
    a, b = g.probes(), o.probes()
    assert a.shape == b.shape == (30, 8, 6)
    assert rel_l2(a, b) <= TOL
    assert np.all(a[:, 0, :] == 0)  # (Nx-1, Ny-1, Nz-1) lies outside every staggered extent


def test_snapshot_cadence_and_values(engine):
    """Snapshots at t % every == 0 after the E update (two_dim_pml.cc:184, three_dim_pml.cc:279)."""
    from luxum_gb300 import Sim
    from oracle.oracle import OracleSim

    p, steps, boxes = cases.build("3d_pml_axis")
    g = Sim(p)
    got = {}

    def cb(t, comp, arr):
        got[(t, comp)] = arr

    g.set_snapshots(7, (1 << 2) | (1 << 6), cb)
    g.step(22)
    g.sync()
    assert sorted(got) == [(0, 2), (0, 6), (7, 2), (7, 6), (14, 2), (14, 6), (21, 2), (21, 6)]
    o = OracleSim(p, threads=4)
    o.step(15)  # state after the step with t = 14
    assert rel_l2(got[(14, 2)], o.field(2)) <= TOL
    ez, ey, ex = o.field(2), o.field(1), o.field(0)
    et = np.zeros(o.shape(2))
    nx, ny, nz = p.Nx, p.Ny, p.Nz
    et[: nx - 1, : ny - 1, : nz - 1] = (ez[: nx - 1, : ny - 1, : nz - 1] ** 2 + ey[: nx - 1, : ny - 1, : nz - 1] ** 2
                                        + ex[: nx - 1, : ny - 1, : nz - 1] ** 2)
    assert rel_l2(got[(14, 6)], et) <= TOL


def test_write_read_reset(engine):
    from luxum_gb300 import Sim

    p, steps, boxes = cases.build("planar_pml_axis")
    g = Sim(p)
    rng = np.random.default_rng(1)
    for c in (1, 3, 5):
        a = rng.standard_normal(g.shape(c))
        g.set_field(c, a)
        assert np.array_equal(g.field(c), a)
    g.step(3)
    assert g.t == 3
    g.reset()
    assert g.t == 0
    for c in (1, 3, 5):
        assert not np.any(g.field(c))


def test_blowup_is_reported(engine):
    """A non-finite field is reported as LX_ERR_BLOWUP after the step, not silently kept."""
    from luxum_gb300 import LuxumError, Sim

    p, steps, boxes = cases.build("planar_oblique")
    g = Sim(p)
    a = np.zeros(g.shape(1))
    a[10, 0, 10] = np.inf
    g.set_field(1, a)
    with pytest.raises(LuxumError) as ei:
        g.step(2)
    assert ei.value.status == 5


@pytest.mark.parametrize("scale", ["mixed", "tiny", "huge", "sparse_denormal", "near_equal", "planes"])
def test_max_monitor_equals_etotal_max(engine, scale):
    """The max|E|^2 monitor (a block reduction on bit patterns, then atomicMax) equals, bit for
    bit, the maximum of the |E|^2 array a twin keeps: values from subnormal to huge, near-equal
    values and values constant over planes."""
    from luxum_gb300 import ETOTAL, Sim

    p, _, _ = cases.build("3d_pml_axis")
    rng = np.random.default_rng({"mixed": 1, "tiny": 2, "huge": 3, "sparse_denormal": 4, "near_equal": 5, "planes": 6}[scale])
    a, b = Sim(p), Sim(p)
    for c in range(6):
        shp = a.shape(c)
        if scale == "mixed":  # magnitudes 1e-300 .. 1e30 side by side
            v = rng.standard_normal(shp) * 10.0 ** rng.uniform(-300, 30, shp)
        elif scale == "tiny":  # squares below float's normal range
            v = rng.standard_normal(shp) * 1e-25
        elif scale == "huge":  # squares beyond float's range
            v = rng.standard_normal(shp) * 1e25
        elif scale == "near_equal":  # every cell within 1e-9 of the others
            v = 1.0 + rng.standard_normal(shp) * 1e-9
        elif scale == "planes":  # one value per x plane, as in a plane wave
            v = np.broadcast_to(rng.standard_normal((shp[0], 1, 1)), shp).copy()
        else:  # zeros with a few subnormal doubles
            v = np.zeros(shp)
            idx = tuple(rng.integers(0, n, 5) for n in shp)
            v[idx] = 1e-310
        a.set_field(c, v)
        b.set_field(c, v)
    got = []
    b.set_snapshots(1, 1 << ETOTAL, lambda t, comp, arr: got.append(arr.max()))
    for _ in range(3):
        a.step(1)
        b.step(1)
        b.sync()
        assert a.max_e2() == b.max_e2() == got[-1]


@pytest.mark.parametrize("name", ["planar_pml_axis", "3d_pml_axis"])
def test_max_series_matches_oracle(engine, name):
    """monitor_every = 1 with a device series: every step's max|E|^2, read once per chunk."""
    from luxum_gb300 import Sim
    from oracle.oracle import OracleSim

    p, steps, boxes = cases.build(name)
    p.monitor_every = 1
    g, o = Sim(p), OracleSim(p, threads=4)
    for lo, hi, eps in boxes:
        g.set_eps_box(lo, hi, eps)
        o.set_eps_box(lo, hi, eps)
    g.set_max_series(25)
    got_t, got_v = [], []
    for _ in range(3):
        g.step(20)
        t, v = g.max_series()
        got_t += list(t)
        got_v += list(v)
    assert got_t == list(range(60))
    for t in range(60):
        o.step(1)
        assert got_v[t] == pytest.approx(o.max_e2(), rel=1e-11, abs=1e-300), t
    assert got_v[-1] == g.max_e2()


@pytest.mark.parametrize("shape", [(200, 7, 9), (7, 150, 9), (9, 7, 260), (40, 40, 3)])
@pytest.mark.parametrize("pml_cells", [0, 2])
def test_elongated_and_thin_grids(engine, shape, pml_cells):
    """Extreme aspect ratios, slabs that cover most of an axis, and tiles that are mostly
    outside the grid: the block-level fast path and slab tests at their edges."""
    from luxum_gb300 import Sim
    from oracle.oracle import OracleSim

    nx, ny, nz = shape
    kw = dict(isPlanar=0, Nx=nx, Ny=ny, Nz=nz, usePS=1, Nx_source=nx // 2, Ny_source=ny // 2, Nz_source=nz // 2 - 1,
              amp_source=1.0, omega_source=3.0e11)
    if pml_cells:
        kw.update(cases.pml(pml_cells, kappa=3.0, a_max=0.0))
    p = cases.make(**kw)
    g, o = Sim(p), OracleSim(p, threads=4)
    g.step(60)
    o.step(60)
    _compare(g, o, f"{shape} pml {pml_cells}")
