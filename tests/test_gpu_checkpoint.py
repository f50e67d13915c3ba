"""Checkpoint / resume (lx_sim_save, lx_sim_load): a run resumed from a checkpoint must go
on bit for bit as the run that wrote it, in every precision, CPML psi and DFT accumulators
included; the fields in the file are those the snapshot files hold."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

W = 2 * np.pi * np.linspace(3e10, 1.5e11, 4)


def _make(name, precision):
    from luxum_gb300 import Sim

    p, _, boxes = cases.build(name)
    p.precision = precision
    s = Sim(p)
    for lo, hi, eps in boxes:
        s.set_eps_box(lo, hi, eps)
    plane = s.add_dft_plane(0, 20, W, every=3)
    return s, plane


@pytest.mark.parametrize("precision", [0, 1, 2])
@pytest.mark.parametrize("name", ["3d_pml_axis", "planar_pml_axis", "3d_pml_pulse_nonuniform"])
def test_resume_is_bit_exact(engine, tmp_path, name, precision):
    from luxum_gb300 import hdf5_read

    a, pa = _make(name, precision)
    a.step(41)
    path = tmp_path / "ck.h5"
    a.save(path)
    ez_saved = a.field(1 if a.p.isPlanar else 2)
    a.step(29)
    b, pb = _make(name, precision)
    b.step(7)  # whatever state b had is replaced
    b.load(path)
    assert b.t == 41
    assert np.array_equal(hdf5_read(path, "Ey" if a.p.isPlanar else "Ez"), ez_saved)
    b.step(29)
    assert b.t == a.t == 70
    for c in range(6):
        if np.prod(a.shape(c)):
            assert np.array_equal(a.field(c), b.field(c)), c
    assert np.array_equal(a.dft(pa), b.dft(pb))
    assert a.max_e2() == b.max_e2()


def test_load_rejects_other_parameters(engine, tmp_path):
    from luxum_gb300 import LuxumError

    a, _ = _make("3d_pml_axis", 0)
    a.step(3)
    a.save(tmp_path / "ck.h5")
    b, _ = _make("3d_pml_axis", 1)  # other precision
    with pytest.raises(LuxumError):
        b.load(tmp_path / "ck.h5")
    c, _ = _make("3d_oblique", 0)  # other grid
    with pytest.raises(LuxumError):
        c.load(tmp_path / "ck.h5")
