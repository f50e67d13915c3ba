"""Parameter sets shared by the tests: small grids of every reference driver.

Each case names the reference driver it exercises (maxwell::solve dispatch,
maxwell.cc:157-174): planar/3-D x PML/no-PML, with TF/SF plane waves along axes and
oblique, dielectric blocks, point sources and non-uniform spacing.
"""
from __future__ import annotations

import math

import numpy as np

from luxum_gb300._ffi import Params

PW_SIGMA = pow(10, -4) / 0.5  # maxwell.cc:71


def make(**kw) -> Params:
    p = Params()
    d = dict(dx=1e-3, dy=1e-3, dz=1e-3, S=0.5, npX=1, npY=1, n_threads=1, pw_sigma=PW_SIGMA, sigma=0.65, sigma_m=3,
             kappa=1, a_m=1, src_tw=1.0, precision=0, cpml_mode=0, source_kind=0, monitor_every=0)
    d.update(kw)
    for k, v in d.items():
        setattr(p, k, v)
    return p


def pw(k, E, box, off=30.0):
    """Plane-wave keys: direction k, polarisation E, total-field box ((x1,x2),(y1,y2),(z1,z2))."""
    (x1, x2), (y1, y2), (z1, z2) = box
    return dict(usePW=1, kx_pw=k[0], ky_pw=k[1], kz_pw=k[2], Ex_pw=E[0], Ey_pw=E[1], Ez_pw=E[2], off_pw=off,
                x1_pw=x1, x2_pw=x2, y1_pw=y1, y2_pw=y2, z1_pw=z1, z2_pw=z2)


def pml(cells, kappa=5.0, a_max=0.05, m=3, ratio=0.65, a_m=1.0, dx=1e-3):
    return dict(usePML=1, d_pml=cells * dx, kappa=kappa, a_max=a_max, sigma_m=m, sigma=ratio, a_m=a_m)


S3 = 1 / math.sqrt(3)
S2 = 1 / math.sqrt(2)

# name -> (params kwargs, steps, eps boxes [(lo, hi, eps_r)])
CASES = {
    # solve_planar_pml (two_dim_pml.cc): the small form of the 512^2 CPML/TF-SF/dielectric config
    "planar_pml_axis": (dict(isPlanar=1, Nx=64, Ny=1, Nz=64, **pw((1, 0, 0), (0, 1, 0), ((12, 51), (0, 0), (12, 51))),
                             **pml(8)), 120, [((28, 0, 28), (36, 1, 36), 10.89)]),
    # solve_planar (two_dim.cc), oblique incidence, non-square grid
    "planar_oblique": (dict(isPlanar=1, Nx=48, Ny=1, Nz=40, **pw((0.6, 0, 0.8), (0, 1, 0), ((10, 37), (0, 0), (9, 30)))),
                       90, []),
    # solve_planar_pml with the textbook CPML sign, oblique
    "planar_pml_std_oblique": (dict(isPlanar=1, Nx=56, Ny=1, Nz=50, cpml_mode=1,
                                    **pw((S2, 0, S2), (0, 1, 0), ((11, 44), (0, 0), (10, 39))), **pml(7)), 100, []),
    # solve3d_pml (three_dim_pml.cc): the small form of the 256^3 config (x-directed wave, dielectric cube)
    "3d_pml_axis": (dict(isPlanar=0, Nx=34, Ny=30, Nz=36, **pw((1, 0, 0), (0, 0, 1), ((9, 24), (8, 21), (9, 26))),
                         **pml(6, kappa=15, a_max=0.0)), 60, [((14, 12, 15), (20, 18, 21), 6.0)]),
    # solve3d (three_dim.cc) with the fixture's oblique direction k = (1,1,1)/sqrt3
    "3d_oblique": (dict(isPlanar=0, Nx=30, Ny=30, Nz=30,
                        **pw((S3, S3, S3), (S2, 0, -S2), ((8, 21), (8, 21), (8, 21)), off=0.0)), 50, []),
    # solve3d_pml with a y-directed wave and a_max > 0 (reference b sign)
    "3d_pml_y_amax": (dict(isPlanar=0, Nx=28, Ny=32, Nz=26, **pw((0, 1, 0), (1, 0, 0), ((7, 20), (8, 23), (7, 18))),
                           **pml(5, kappa=5, a_max=0.05)), 50, []),
    # solve3d_pml with the reference's hard CW point source (int amp/omega) and no plane wave
    "3d_pml_point_cw": (dict(isPlanar=0, Nx=26, Ny=24, Nz=28, usePS=1, Nx_source=13, Ny_source=11, Nz_source=14,
                             amp_source=3.0, omega_source=2.0e9, **pml(5, kappa=15, a_max=0.0)), 60, []),
    # extension: pulsed additive source, non-uniform spacing, z-directed wave
    "3d_pml_pulse_nonuniform": (dict(isPlanar=0, Nx=26, Ny=22, Nz=30, dx=1e-3, dy=1.25e-3, dz=0.8e-3, usePS=1,
                                     source_kind=1, Nx_source=12, Ny_source=10, Nz_source=15, amp_source=1.0,
                                     omega_source=3.0e11, src_t0=20.0, src_tw=8.0,
                                     **pw((0, 0, 1), (0, 1, 0), ((7, 18), (6, 15), (8, 21))), **pml(5, kappa=5)), 55, []),
}


def build(name: str):
    kw, steps, boxes = CASES[name]
    return make(**kw), steps, boxes


def rel_l2(a: np.ndarray, b: np.ndarray) -> float:
    nb = float(np.linalg.norm(b))
    na = float(np.linalg.norm(a - b))
    if nb == 0.0:
        return 0.0 if na == 0.0 else float("inf")
    return na / nb


def field_errors(get_a, get_b, shapes):
    """Per-component error relative to the norm of its field group (E or H).

    A component can be pure cancellation noise (e.g. Hz of a z-directed point source is
    ~1e-16 of |H|); measuring it against its own norm would be meaningless, so every
    component's error is taken relative to ||E|| or ||H|| of the reference solution.
    Returns {component: error}.
    """
    out = {}
    for group in ((0, 1, 2), (3, 4, 5)):
        comps = [c for c in group if np.prod(shapes[c]) > 0]
        bs = {c: get_b(c) for c in comps}
        gn = float(np.sqrt(sum(np.linalg.norm(b) ** 2 for b in bs.values())))
        for c in comps:
            d = float(np.linalg.norm(get_a(c) - bs[c]))
            out[c] = d / gn if gn > 0 else (0.0 if d == 0 else float("inf"))
    return out
