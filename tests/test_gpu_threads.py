"""Distinct handles from distinct host threads (the ABI's threading contract): each thread
creates, steps and reads its own handle at the same time as the others; every result equals
the same simulation run alone."""
import threading

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

NAMES = ["planar_pml_axis", "3d_pml_axis", "3d_oblique", "planar_oblique", "3d_pml_point_cw", "3d_pml_y_amax"]


def _run(name, precision):
    from luxum_gb300 import Sim

    p, steps, boxes = cases.build(name)
    p.precision = precision
    s = Sim(p)
    for lo, hi, eps in boxes:
        s.set_eps_box(lo, hi, eps)
    s.step(steps)
    out = [s.field(c) if np.prod(s.shape(c)) else None for c in range(6)] + [s.max_e2()]
    s.close()
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_distinct_handles_in_threads(engine, precision):
    alone = {n: _run(n, precision) for n in NAMES}
    got, errors = {}, []

    def work(n):
        try:
            got[n] = _run(n, precision)
        except Exception as e:  # reported below
            errors.append((n, e))

    threads = [threading.Thread(target=work, args=(n,)) for n in NAMES * 2]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    for n in NAMES:
        for a, b in zip(alone[n], got[n]):
            if a is None:
                continue
            assert np.array_equal(a, b), n
