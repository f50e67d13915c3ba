"""Regenerates the golden fixtures from the oracle: python tests/golden/make_golden.py

Each fixture holds, for one small case of tests/cases.py, the oracle's state after the
case's step count: full fields for the planar case, and for 3-D cases every third cell of
each component plus per-component sum and L2 norm of the whole array, the max|E|^2
monitor and an 8-probe series.  manifest.json records the cases and the generator.
"""
import json
import os
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
sys.path.insert(0, str(HERE.parent))

import cases  # noqa: E402
from oracle.oracle import OracleSim  # noqa: E402

GOLDEN_CASES = ["planar_pml_axis", "3d_pml_axis", "3d_oblique", "3d_pml_point_cw"]


def probe_points(p):
    rng = np.random.default_rng(2026)
    return np.stack([rng.integers(0, n, 8) for n in (p.Nx, p.Ny if not p.isPlanar else 1, p.Nz)], axis=1)


def run(name):
    p, steps, boxes = cases.build(name)
    o = OracleSim(p, threads=os.cpu_count() or 1)
    for lo, hi, eps in boxes:
        o.set_eps_box(lo, hi, eps)
    ijk = probe_points(p)
    o.set_probes(ijk, steps)
    o.step(steps)
    out = {"max_e2": np.array(o.max_e2()), "probes": o.probes(), "probe_ijk": ijk.astype(np.int32)}
    for c in range(6):
        shp = o.shape(c)
        if np.prod(shp) == 0:
            continue
        f = o.field(c)
        out[f"sum{c}"] = np.array(f.sum())
        out[f"norm{c}"] = np.array(np.linalg.norm(f))
        out[f"f{c}"] = f if p.isPlanar else f[::3, ::3, ::3]
    return p, steps, out


def main():
    manifest = {"generator": "tests/golden/make_golden.py", "source": "oracle/luxum_oracle.c (FP64, no FMA)",
                "cases": {}}
    for name in GOLDEN_CASES:
        p, steps, out = run(name)
        np.savez_compressed(HERE / f"{name}.npz", **out)
        manifest["cases"][name] = {"steps": steps, "params": {k: v for k, v in p.as_dict().items()},
                                   "stored": "full fields" if p.isPlanar else "every 3rd cell + sum + L2 norm"}
    (HERE / "manifest.json").write_text(json.dumps(manifest, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
