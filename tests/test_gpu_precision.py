"""FP32 and FP16-storage variants against the FP64 oracle.

Stated tolerances (relative L2 per field component, after the case's step count):
  FP32 (fields, psi and coefficients in FP32; profiles and TF/SF tables evaluated in FP64):
       <= 1e-4 (spec bar for the FP32 form)
  FP16 storage / FP32 compute (E, H stored as binary16):
       <= 3e-2 (stated error of the storage format; no bar in the benchmark spec)
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
    worst = 0.0
    for c in range(6):
        if np.prod(o.shape(c)) == 0:
            continue
        b = o.field(c)
        if np.linalg.norm(b) < 1e-9 * max(np.linalg.norm(o.field(k)) for k in range(3) if np.prod(o.shape(k))):
            continue  # components that stay ~0 (cross-polarised leakage) have no meaningful relative error
        worst = max(worst, rel_l2(g.field(c), b))
    assert worst <= TOL[prec], f"{name} precision {prec}: rel-L2 {worst:.3e}"
    assert worst > 0  # it really ran in reduced precision
