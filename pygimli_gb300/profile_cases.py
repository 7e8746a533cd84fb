"""Single workloads for kernel profiling (``ncu`` launch lists and captures):

    python -m pygimli_gb300.profile_cases complex [box_3d_probe|box_3d|line_2d] [fp64|mixed]
    python -m pygimli_gb300.profile_cases refine  [box_3d_probe|box_3d|line_2d]

``complex``: one complex-resistivity response (-10 mrad on the workload's
amplitudes) and its complex Jacobian; ``refine``: the GPU H2 refinement of
the workload's mesh, twice.  Each prints one line with the wall time.
"""
from __future__ import annotations

import sys
import time

import numpy as np


def _workload(name):
    from . import synthetic
    if name == "line_2d":
        return synthetic.line_2d()
    return synthetic.box_3d(scheme="inline" if name == "box_3d_probe" else "full")


def complex_case(name="box_3d_probe", precision="mixed"):
    from .ert import ERTModelling
    mesh, data, rho = _workload(name)
    fop = ERTModelling(precision=precision)
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    fop.setComplex(True)
    z = rho * np.exp(-0.01j)
    t0 = time.perf_counter()
    fop.response(z)
    fop.createJacobian(z)
    st = fop.stats()
    print(f"complex {name} {precision}: {time.perf_counter() - t0:.3f} s, COCG iterations {st['iterations']}, "
          f"columns finished in FP64 {st['stalled_columns']}")


def refine_case(name="box_3d_probe"):
    from . import refine
    mesh = _workload(name)[0]
    for _ in range(2):
        t0 = time.perf_counter()
        h = refine.createH2(mesh, 0)
    print(f"refine {name}: H2 of {mesh.cellCount()} cells -> {h.cellCount()} in {time.perf_counter() - t0:.4f} s")


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "complex"
    args = sys.argv[2:]
    if what == "complex":
        complex_case(*args)
    elif what == "refine":
        refine_case(*args)
    else:
        raise SystemExit(f"unknown case {what}")
