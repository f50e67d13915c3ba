"""Failures of the snapshot writer reach the caller as LX_ERR_IO, with the file's path.

The reference writes snapshots synchronously and exits on a failed open
(fileio.cc:133-137); here files are written by a host thread while the time loop runs, so a
failed write must surface at the next call that waits for the writer (lx_sim_sync, or the
next lx_sim_step) instead of being lost.  The failures are made on the host: a directory
that does not exist, and /dev/full, which accepts the open and fails every flushed write
with ENOSPC.  No GPU fault is involved.
"""
import os

import pytest

import cases

pytestmark = pytest.mark.gpu

LX_EY = 1
LX_ERR_IO = 6


def _sim():
    from luxum_gb300 import Sim

    p, _, boxes = cases.build("planar_pml_axis")
    s = Sim(p)
    for lo, hi, eps in boxes:
        s.set_eps_box(lo, hi, eps)
    return s


def test_output_in_missing_directory_is_refused(engine, tmp_path):
    from luxum_gb300 import LuxumError

    path = tmp_path / "no_such_dir" / "Ey_data_2d.h5"
    s = _sim()
    with pytest.raises(LuxumError) as e:
        s.set_hdf5_output(10, LX_EY, str(path))
    assert e.value.status == LX_ERR_IO
    assert str(path) in str(e.value)
    s.step(5)  # the handle stays usable
    s.close()


@pytest.mark.skipif(not os.path.exists("/dev/full"), reason="needs /dev/full")
def test_failed_snapshot_write_reaches_the_caller(engine):
    from luxum_gb300 import LuxumError

    s = _sim()
    s.set_hdf5_output(10, LX_EY, "/dev/full")  # the open succeeds; writes fail
    with pytest.raises(LuxumError) as e:
        s.step(25)  # snapshots at t = 0, 10, 20
        s.sync()
    assert e.value.status == LX_ERR_IO
    assert "failed on /dev/full" in str(e.value)  # the flush inside the write's seek, or the write
    # the error is reported once; stepping goes on (the file output stays broken, the fields do not)
    s.sync()
    t = s.t
    s.step(3)
    assert s.t == t + 3
    s.close()
