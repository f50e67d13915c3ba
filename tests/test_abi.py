"""The C ABI (include/luxum.h) on the CPU: exports, parameter defaults, validation, YAML.

No compute call is made here: lx_sim_create validates its parameters before touching the
GPU, so every rejection path runs without one.
"""
import ctypes as C
import math
import pathlib
import re

import pytest

import cases

ROOT = pathlib.Path(__file__).resolve().parent.parent
GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"


def declared_symbols():
    text = (ROOT / "include" / "luxum.h").read_text()
    return sorted(set(re.findall(r"^LX_API\s+[\w\s\*]*?\b(lx_\w+)\s*\(", text, re.M)))


def test_header_declares_api():
    names = declared_symbols()
    assert "lx_sim_create" in names and "lx_sim_step" in names and len(names) >= 20


def test_library_exports_every_declared_symbol(engine):
    for name in declared_symbols():
        assert hasattr(engine, name), name


def test_params_struct_layout_matches_c(oracle_lib):
    from luxum_gb300._ffi import Params

    assert C.sizeof(Params) == oracle_lib.ox_params_size()


def test_param_defaults(engine):
    from luxum_gb300 import params

    p = params()
    assert p.pw_sigma == pow(10, -4) / 0.5  # maxwell.cc:71
    assert (p.npX, p.npY, p.precision, p.cpml_mode, p.source_kind) == (1, 1, 0, 0, 0)


BAD = {
    # reader::checkData (reader.cc:141-162)
    "x_not_divisible": dict(isPlanar=0, Nx=33, Ny=30, Nz=30, npX=2),
    "planar_Ny": dict(isPlanar=1, Nx=30, Ny=3, Nz=30),
    "planar_npY": dict(isPlanar=1, Nx=30, Ny=1, Nz=30, npY=3),
    # index ranges the reference reads out of bounds
    "box_touches_wall": dict(isPlanar=0, Nx=30, Ny=30, Nz=30, **cases.pw((1, 0, 0), (0, 0, 1), ((0, 20), (5, 20), (5, 20)))),
    "box_past_wall": dict(isPlanar=1, Nx=30, Ny=1, Nz=30, **cases.pw((1, 0, 0), (0, 1, 0), ((5, 29), (0, 0), (5, 20)))),
    "k_parallel_E": dict(isPlanar=0, Nx=30, Ny=30, Nz=30, **cases.pw((1, 0, 0), (1, 0, 0), ((5, 20), (5, 20), (5, 20)))),
    "pml_one_cell": dict(isPlanar=0, Nx=30, Ny=30, Nz=30, **cases.pml(1)),
    "pml_fractional_m": dict(isPlanar=0, Nx=30, Ny=30, Nz=30, **cases.pml(5, m=2.5)),
    "source_z_outside": dict(isPlanar=0, Nx=30, Ny=30, Nz=30, usePS=1, Nx_source=3, Ny_source=3, Nz_source=29),
    "tiny_grid": dict(isPlanar=0, Nx=2, Ny=30, Nz=30),
}


@pytest.mark.parametrize("name", sorted(BAD))
def test_invalid_parameters_rejected_like_oracle(name, engine, oracle_lib):
    from oracle.oracle import OracleError, OracleSim

    p = cases.make(**BAD[name])
    h = C.c_void_p()
    st = engine.lx_sim_create(C.byref(p), C.byref(h))
    assert st == 1, (name, st, engine.lx_last_error(None))
    assert engine.lx_last_error(None)
    with pytest.raises(OracleError) as ei:
        OracleSim(p)
    assert ei.value.status == 1


def test_planar_point_source_unsupported(engine):
    """The reference writes E->Vz in planar mode, which does not exist (vfield.cc:69-71)."""
    p = cases.make(isPlanar=1, Nx=30, Ny=1, Nz=30, usePS=1, Nx_source=5, Nz_source=5)
    h = C.c_void_p()
    assert engine.lx_sim_create(C.byref(p), C.byref(h)) == 2
    assert b"Vz" in engine.lx_last_error(None)


def test_yaml_fixture_2d(engine):
    from luxum_gb300 import read_yaml

    p = read_yaml(GOLDEN / "params_2d.yaml")
    assert (p.isPlanar, p.Nx, p.Ny, p.Nz) == (1, 130, 1, 130)
    assert p.dx == 0.001 and p.dy == 0 and p.S == 0.5 and p.num_timesteps == 300
    assert (p.npX, p.npY, p.n_threads) == (2, 1, 4)
    assert p.usePW == 1 and p.usePS == 0 and p.kx_pw == 1 and p.Ey_pw == 1 and p.off_pw == 40
    assert (p.x1_pw, p.x2_pw, p.z1_pw, p.z2_pw) == (25, 104, 25, 104)
    assert p.usePML == 1 and p.d_pml == 0.02 and p.kappa == 5 and p.a_max == 0.05


def test_reference_parameters_yaml_verbatim(engine):
    """The reference's own parameters.yaml (byte-for-byte copy, UTF-8 BOM, comments and
    trailing commas included) parses as reader::readYAML reads it (reader.cc:68-130) and
    passes checkData: (1002 - 2) % 2 == 0 for the two x ranks (reader.cc:143-159)."""
    from luxum_gb300 import read_yaml

    raw = (GOLDEN / "reference_parameters.yaml").read_bytes()
    assert raw.startswith(b"\xef\xbb\xbf")  # the verbatim file, BOM first
    p = read_yaml(GOLDEN / "reference_parameters.yaml")
    assert (p.isPlanar, p.Nx, p.Ny, p.Nz) == (1, 1002, 1, 1002)
    assert (p.dx, p.dy, p.dz) == (0.001, 0.0, 0.001)
    assert p.S == 0.70710678118 and p.num_timesteps == 2000
    assert (p.npX, p.npY, p.n_threads) == (2, 1, 1)
    assert (p.usePS, p.Nx_source, p.Ny_source, p.Nz_source, p.amp_source, p.omega_source) == (0, 0, 0, 0, 0, 0)
    assert p.usePW == 1 and (p.kx_pw, p.ky_pw, p.kz_pw) == (0.70710678118, 0.0, 0.70710678118)
    assert (p.Ex_pw, p.Ey_pw, p.Ez_pw, p.off_pw) == (0.0, 1.0, 0.0, 50.0)
    assert (p.x1_pw, p.y1_pw, p.z1_pw, p.x2_pw, p.y2_pw, p.z2_pw) == (20, 20, 20, 980, 980, 980)
    assert p.usePML == 0 and p.d_pml == 0.01 and p.sigma == 0.65 and p.sigma_m == 3
    assert (p.kappa, p.a_max, p.a_m) == (15.0, 0.0, 1.0)
    assert p.precision == 0 and p.cpml_mode == 0  # no engine-options document: reference behaviour


def test_reference_parameters_3d_yaml_verbatim(engine):
    """The reference's parameters_3d.yaml, verbatim: a 102^3 oblique plane wave with CPML on a
    2 x 2 rank grid ((102 - 2) % 2 == 0 on both axes)."""
    from luxum_gb300 import read_yaml

    p = read_yaml(GOLDEN / "reference_parameters_3d.yaml")
    assert (p.isPlanar, p.Nx, p.Ny, p.Nz) == (0, 102, 102, 102)
    assert (p.dx, p.dy, p.dz) == (0.001, 0.001, 0.001)
    assert p.S == 0.5773502691896258 and p.num_timesteps == 600
    assert (p.npX, p.npY, p.n_threads) == (2, 2, 1)
    assert p.usePW == 1 and p.kx_pw == p.ky_pw == p.kz_pw == 0.5773502691896258
    assert (p.Ex_pw, p.Ey_pw, p.Ez_pw, p.off_pw) == (0.70710678118, 0.0, -0.70710678118, 0.0)
    assert (p.x1_pw, p.y1_pw, p.z1_pw, p.x2_pw, p.y2_pw, p.z2_pw) == (20, 20, 20, 80, 80, 80)
    assert p.usePML == 1 and p.d_pml == 0.01 and p.sigma == 0.65 and p.sigma_m == 3
    assert (p.kappa, p.a_max, p.a_m) == (15.0, 0.0, 1.0)


def test_yaml_fixture_3d_engine_options(engine):
    from luxum_gb300 import read_yaml

    p = read_yaml(GOLDEN / "params_3d.yaml")
    assert (p.isPlanar, p.Nx, p.Ny, p.Nz) == (0, 66, 66, 66)
    assert math.isclose(p.kx_pw, 1 / math.sqrt(3), rel_tol=1e-12)
    assert p.precision == 1 and p.cpml_mode == 1 and p.monitor_every == 10


@pytest.mark.parametrize("mutation, status", [
    (lambda s: s.replace('"X Length": 130,', ''), 6),           # missing key
    (lambda s: s.replace('"X Length": 130', '"X Length": 1.5e2'), 6),  # not an integer
    (lambda s: s.replace('"usePW": true', '"usePW": maybe'), 6),     # not a boolean
    (lambda s: s.replace('"X Number of Procs": 2', '"X Number of Procs": 3'), 1),  # checkData
    (lambda s: s[: s.index("{   # absorbing layer")], 6),          # four documents only
])
def test_yaml_errors(engine, tmp_path, mutation, status):
    from luxum_gb300 import LuxumError, read_yaml

    src = (GOLDEN / "params_2d.yaml").read_text(encoding="utf-8")
    bad = tmp_path / "parameters.yaml"
    bad.write_text(mutation(src), encoding="utf-8")
    with pytest.raises(LuxumError) as ei:
        read_yaml(bad)
    assert ei.value.status == status


def test_ctypes_structs_match_the_header(tmp_path):
    """Sizes and member offsets of the ABI structs as a C compiler lays them out."""
    import shutil
    import subprocess

    from luxum_gb300 import _ffi

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    structs = {"lx_params": _ffi.Params, "lx_request": _ffi.Request, "lx_server_config": _ffi.ServerConfig,
               "lx_server_stats": _ffi.ServerStats, "lx_info": _ffi.Info, "lx_tune_entry": _ffi.TuneEntry}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "luxum.h"', "int main(void) {"]
    for name, py in structs.items():
        lines.append(f'  printf("{name} %zu\\n", sizeof({name}));')
        for field, _ in py._fields_:
            lines.append(f'  printf("{name}.{field} %zu\\n", offsetof({name}, {field}));')
    lines.append("  return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for name, py in structs.items():
        assert int(got[name]) == C.sizeof(py), name
        for field, _ in py._fields_:
            assert int(got[f"{name}.{field}"]) == getattr(py, field).offset, (name, field)


@pytest.mark.parametrize("precision,two_buffers", [(0, False), (1, True), (2, True)])
def test_device_bytes_counts_the_second_state_buffer(engine, monkeypatch, precision, two_buffers):
    """Planar FP32 / FP16-storage handles keep two copies of E, H and psi (the single-sweep
    step), and so do 3-D ones with LUXUM_SWEEP3=1; lx_params_device_bytes, which the server
    admits requests by, counts both.  FP64 handles keep one.  LUXUM_TWO_SWEEP=1 keeps new float
    handles at one copy."""
    from luxum_gb300 import device_bytes, field_shape

    kw = dict(isPlanar=1, Nx=300, Ny=1, Nz=520, precision=precision, **cases.pml(16))
    p = cases.make(**kw)
    monkeypatch.delenv("LUXUM_TWO_SWEEP", raising=False)
    both = device_bytes(p)
    monkeypatch.setenv("LUXUM_TWO_SWEEP", "1")
    one = device_bytes(p)
    if not two_buffers:
        assert both == one
        return
    # the difference is one copy of Ey, Hx, Hz (padded rows) and of the four planar psi
    # arrays (float): x slabs of Hz and Ey, n x Nzp each; z slabs of Hx and Ey, Nx x n each,
    # with n the packed slab width (at most the 2 x 16 CPML cells)
    tsize = {1: 4, 2: 2}[precision]
    nzp = -(-520 * tsize // 128) * 128 // tsize
    fields = 3 * 300 * nzp * tsize
    per_cell_of_width = (2 * nzp + 2 * 300) * 4
    psi = both - one - fields
    assert psi % per_cell_of_width == 0 and 16 <= psi // per_cell_of_width <= 32
    # 3-D: one copy, unless the single-sweep kernel is asked for (then a second copy of the six
    # components; no CPML here)
    p3 = cases.make(isPlanar=0, Nx=40, Ny=40, Nz=40, precision=precision)
    monkeypatch.delenv("LUXUM_TWO_SWEEP", raising=False)
    monkeypatch.delenv("LUXUM_SWEEP3", raising=False)
    one3 = device_bytes(p3)
    monkeypatch.setenv("LUXUM_SWEEP3", "1")
    nzp3 = -(-40 * tsize // 128) * 128 // tsize
    assert device_bytes(p3) - one3 == 6 * 40 * 40 * nzp3 * tsize
    monkeypatch.setenv("LUXUM_TWO_SWEEP", "1")
    assert device_bytes(p3) == one3
