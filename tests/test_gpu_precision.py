"""FP32 and FP16-storage variants against the FP64 oracle.

Stated tolerances (relative L2 per field component, relative to its field group's norm as
in cases.field_errors, after the case's step count):
  FP32 (fields, psi and coefficients in FP32; profiles and TF/SF positions in FP64, the
       TF/SF exponential in FP32): <= 1e-4, the bound the FP32 form is held to
  FP16 storage / FP32 compute (E, H stored as binary16):
       <= 3e-2 (the storage format's own error; the form is held to no tighter bound)
"""
import numpy as np
import pytest

import cases
from cases import rel_l2

pytestmark = pytest.mark.gpu

TOL = {1: 1e-4, 2: 3e-2}


@pytest.mark.parametrize("prec", [1, 2])
@pytest.mark.parametrize("name", ["planar_pml_axis", "3d_pml_axis", "3d_oblique", "3d_pml_pulse_nonuniform"])
def test_reduced_precision_error(name, prec, engine):
    from luxum_gb300 import Sim
    from oracle.oracle import OracleSim

    p, steps, boxes = cases.build(name)
    o = OracleSim(p, threads=4)
    p.precision = prec
    g = Sim(p)
    for lo, hi, eps in boxes:
        g.set_eps_box(lo, hi, eps)
        o.set_eps_box(lo, hi, eps)
    g.step(steps)
    o.step(steps)
    errs = cases.field_errors(g.field, o.field, {c: o.shape(c) for c in range(6)})
    worst = max(errs.values())
    assert worst <= TOL[prec], f"{name} precision {prec}: rel-L2 {worst:.3e}"
    assert worst > 0  # it really ran in reduced precision
