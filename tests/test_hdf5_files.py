"""The HDF5 files the engine writes (lx_hdf5_write, the snapshot writer's format) on the CPU:
checked by a reader written from the format specification (tests/hdf5_spec.py) and by the
engine's own reader, for the dataset names, shapes and values fileio.cc:143-212 produces."""
import numpy as np
import pytest

from hdf5_spec import Spec


def _write(path, datasets):
    from luxum_gb300 import hdf5_write

    hdf5_write(path, datasets)


@pytest.mark.parametrize("n", [1, 3, 17, 40])
def test_spec_reader_opens_engine_files(engine, tmp_path, n):
    rng = np.random.default_rng(n)
    shape = (5, 1, 7) if n % 2 else (4, 6, 3)
    data = {f"t={10 * q}": rng.standard_normal(shape) for q in range(n)}
    path = tmp_path / "snap.h5"
    _write(path, data)
    spec = Spec(path)
    assert set(spec.entries()) == set(data)  # every dataset reachable from the root group
    for name, a in data.items():
        assert np.array_equal(spec.dataset(name), a), name


def test_engine_reader_round_trip(engine, tmp_path):
    from luxum_gb300 import hdf5_read

    rng = np.random.default_rng(7)
    data = {"data": rng.standard_normal((9, 8, 7)), "t=0": np.zeros((9, 8, 7)), "t=250": rng.random((9, 8, 7))}
    path = tmp_path / "m.h5"
    _write(path, data)
    for name, a in data.items():
        assert np.array_equal(hdf5_read(path, name), a)


def test_engine_reader_errors(engine, tmp_path):
    from luxum_gb300 import LuxumError, hdf5_read

    path = tmp_path / "m.h5"
    _write(path, {"data": np.ones((2, 2, 2))})
    with pytest.raises(LuxumError):
        hdf5_read(path, "missing")
    with pytest.raises(LuxumError):
        hdf5_read(tmp_path / "absent.h5", "data")
    bad = tmp_path / "bad.h5"
    bad.write_bytes(b"not an hdf5 file" * 8)
    with pytest.raises(LuxumError):
        hdf5_read(bad, "data")
