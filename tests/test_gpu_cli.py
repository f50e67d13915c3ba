"""The `luxum` command line end to end (main.cc:53-72): parameters.yaml in the working
directory, the driver maxwell::solve picks, its HDF5 file out, one "t: ..., max: ..." line
per step.  Every dataset the CLI writes is compared with the oracle at the same step, and
the printed stream follows the drivers: the line of step t carries the max left by step t-1
(two_dim_pml.cc:135-141), 0 at t = 0.
"""
import pathlib
import re
import shutil
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = pathlib.Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"


def _run(cwd, *args):
    exe = ROOT / "luxum_gb300" / "luxum"
    r = subprocess.run([str(exe), *args], cwd=cwd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return [(int(t), float(m)) for t, m in re.findall(r"^t: (\d+), max: (\S+)$", r.stdout, re.M)]


def _close(a, b, tol=1e-12):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) <= tol * n if n > 0 else np.array_equal(a, b)


def test_cli_planar_pml(engine, tmp_path):
    """solve_planar_pml: Ey_data_2d.h5 with Ey at t % 10 == 0 (two_dim_pml.cc:184)."""
    from luxum_gb300 import EY, hdf5_read, read_yaml
    from oracle.oracle import OracleSim

    shutil.copy(GOLDEN / "params_2d.yaml", tmp_path / "parameters.yaml")
    lines = _run(tmp_path)
    p = read_yaml(tmp_path / "parameters.yaml")
    assert [t for t, _ in lines] == list(range(p.num_timesteps))
    o = OracleSim(p, threads=4)
    assert lines[0][1] == 0.0
    for t in range(p.num_timesteps):
        o.step(1)
        if t + 1 < p.num_timesteps:  # printed with %g
            assert lines[t + 1][1] == pytest.approx(o.max_e2(), rel=1e-5, abs=1e-300), t
        if t % 10 == 0:
            assert _close(hdf5_read(tmp_path / "Ey_data_2d.h5", f"t={t}")[:, 0, :], o.field(EY)[:, 0, :]), t


def test_cli_3d_pml_with_material_files(engine, tmp_path):
    """solve3d_pml: Cb from airplane_100_{x,y,z}.h5, |E|^2 into Ez_data.h5 every 3 steps
    (three_dim_pml.cc:109-128, :279)."""
    from luxum_gb300 import ETOTAL, hdf5_read, hdf5_write, read_yaml
    from oracle.oracle import OracleSim

    text = (GOLDEN / "params_3d.yaml").read_text()
    text = text[: text.rindex("---")]  # drop the engine-options document: FP64, reference CPML
    text = text.replace('"Number of timesteps": 200', '"Number of timesteps": 31')
    (tmp_path / "parameters.yaml").write_text(text)
    p = read_yaml(tmp_path / "parameters.yaml")
    o = OracleSim(p, threads=4)
    rng = np.random.default_rng(11)
    for c, name in enumerate("xyz"):
        F = (rng.random(o.shape(c)) < 0.1) * 5e-6 * rng.random(o.shape(c))
        hdf5_write(tmp_path / f"airplane_100_{name}.h5", {"data": F})
        o.set_material(c, F, 1e6)
    lines = _run(tmp_path, "--print-every", "1")
    assert len(lines) == 31
    for t in range(31):
        o.step(1)
        if t + 1 < 31:
            assert lines[t + 1][1] == pytest.approx(o.max_e2(), rel=1e-5, abs=1e-300), t
        if t % 3 == 0:
            assert _close(hdf5_read(tmp_path / "Ez_data.h5", f"t={t}"), o.field(ETOTAL)), t


def test_cli_missing_material_fails_unless_waived(engine, tmp_path):
    text = (GOLDEN / "params_3d.yaml").read_text()
    text = text[: text.rindex("---")].replace('"Number of timesteps": 200', '"Number of timesteps": 3')
    (tmp_path / "parameters.yaml").write_text(text)
    exe = ROOT / "luxum_gb300" / "luxum"
    r = subprocess.run([str(exe)], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode != 0 and "airplane_100_x.h5" in r.stderr
    assert len(_run(tmp_path, "--no-material")) == 3
    assert (tmp_path / "Ez_data.h5").exists()


def test_cli_reference_parameters_yaml(engine, tmp_path):
    """The reference's own parameters.yaml, unmodified (byte-for-byte copy): solve_planar on
    1002 x 1002 without CPML, an oblique TF/SF wave, 2000 steps, two x ranks in the file (one
    GPU here).  Ey_data_2d.h5 holds Ey at t % 20 == 0 from t = 100 (two_dim.cc:140), and the
    printed line of step t carries the max of step t itself (two_dim.cc:126-137).  Every
    dataset is compared with the oracle at 1e-12."""
    import os

    from luxum_gb300 import EY, hdf5_read, read_yaml
    from oracle.oracle import OracleSim

    shutil.copy(GOLDEN / "reference_parameters.yaml", tmp_path / "parameters.yaml")
    lines = _run(tmp_path)
    p = read_yaml(tmp_path / "parameters.yaml")
    assert [t for t, _ in lines] == list(range(2000))
    o = OracleSim(p, threads=os.cpu_count() or 1)
    checked = 0
    for t in range(2000):
        o.step(1)
        assert lines[t][1] == pytest.approx(o.max_e2(), rel=1e-5, abs=1e-300), t
        if t % 20 == 0 and t >= 100:
            assert _close(hdf5_read(tmp_path / "Ey_data_2d.h5", f"t={t}")[:, 0, :], o.field(EY)[:, 0, :]), t
            checked += 1
    assert checked == 95 and lines[-1][1] > 0


def test_cli_reference_parameters_3d_yaml(engine, tmp_path):
    """The reference's parameters_3d.yaml, unmodified: solve3d_pml on 102^3 with an oblique
    wave, 600 steps.  The airplane_100_*.h5 material files that driver reads are not in the
    reference repository, so the run waives them (--no-material: vacuum, which is also what
    the oracle runs).  |E|^2 goes to Ez_data.h5 every 3 steps (three_dim_pml.cc:279); one
    dataset in 33 is compared with the oracle, and every printed max.

    The file runs at the 3-D Courant limit (S = 1/sqrt 3) in vacuum: once the pulse has left
    the total-field box (t ~ 280), |E|^2 is only the box faces' cancellation residue, some
    1e-3 of its peak, and the relative error of that residue is no measure of the update.  So
    each dataset's difference is bounded by 1e-12 of the largest |E|^2 norm the run has had
    so far; up to t = 264 that is also 1e-12 of the dataset's own norm, and is checked too."""
    import os

    from luxum_gb300 import ETOTAL, hdf5_read, read_yaml
    from oracle.oracle import OracleSim

    shutil.copy(GOLDEN / "reference_parameters_3d.yaml", tmp_path / "parameters.yaml")
    lines = _run(tmp_path, "--no-material")
    p = read_yaml(tmp_path / "parameters.yaml")
    assert [t for t, _ in lines] == list(range(600))
    o = OracleSim(p, threads=os.cpu_count() or 1)
    assert lines[0][1] == 0.0
    checked, peak = 0, 0.0
    for t in range(600):
        o.step(1)
        if t + 1 < 600:
            assert lines[t + 1][1] == pytest.approx(o.max_e2(), rel=1e-5, abs=1e-300), t
        if t % 33 == 0:
            a, b = hdf5_read(tmp_path / "Ez_data.h5", f"t={t}"), o.field(ETOTAL)
            peak = max(peak, float(np.linalg.norm(b)))
            d = float(np.linalg.norm(a - b))
            assert d <= 1e-12 * peak, (t, d / peak)
            if t <= 264:
                assert _close(a, b), t
            checked += 1
    assert checked == 19 and o.max_e2() > 0
