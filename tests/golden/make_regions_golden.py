"""Generate tests/golden/regions.npz with the reference's own RegionManager
(core/src/regionManager.cpp, compiled into oracle/_ref/libgimli_ref.so by
oracle/Makefile, driven through oracle/ref_driver.py).

Run from the repository root after ``make -C oracle``:

    python tests/golden/make_regions_golden.py

Meshes from the project's generators get region markers by position (1
outside the parameter box, 2 inside, 3 and 4 two blocks); each case sets
region flags the way pyGIMLi's MeshModelling does (lowest region background
unless stated, then background / single / fixed-value regions) and stores
the reference's renumbered cell markers, parameter count and para-domain
cell count, and its constraint matrix (RegionManager::fillConstraints) as
(row, column, value) triplets with its shape.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_driver as R  # noqa: E402
from pygimli_gb300.mesh import Mesh, create_box_mesh_3d, create_para_mesh_2d  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "regions.npz")


def region_mesh(dim):
    if dim == 2:
        m = create_para_mesh_2d(np.arange(9.0), para_dx=0.5, para_depth=3.0)
        lo, hi = (0.0, -3.0), (8.0, 0.0)
    else:
        m = create_box_mesh_3d(np.array([(x, y) for x in (0.0, 2.0, 4.0) for y in (0.0, 2.0)]), h=1.0,
                               para_margin=(2, 2), para_depth=3.0, outer=30.0, growth=2.0, depth_growth=2.0)
        lo, hi = (0.0, 0.0, -3.0), (4.0, 2.0, 0.0)
    c = m.cellCenters()[:, :dim]
    inside = np.all((c >= np.array(lo) - 1e-9) & (c <= np.array(hi) + 1e-9), axis=1)
    mk = np.where(inside, 2, 1)
    mk[inside & (c[:, 0] < 2.0) & (c[:, dim - 1] > -1.5)] = 3
    mk[inside & (c[:, 0] > 6.0 if dim == 2 else c[:, 0] > 3.0)] = 4
    return Mesh(dim, m.nodes, m.cells, mk.astype(np.int32), m.node_markers, m.boundaries, m.boundary_markers,
                m.boundary_cells)


CASES = [
    {"name": "default", "default_background": True},
    {"name": "single3", "default_background": True, "single": [3]},
    {"name": "fix3", "default_background": True, "fix": {"3": 50.0}},
    {"name": "bg4_single2", "default_background": False, "background": [4], "single": [2]},
    {"name": "no_background", "default_background": False},
]


def main():
    out = {}
    for dim in (2, 3):
        m = region_mesh(dim)
        out[f"markers_{dim}d"] = m.cell_markers
        rm = R.RefMesh(m)
        for c in CASES:
            fix = {int(k): v for k, v in c.get("fix", {}).items()}
            args = (c["default_background"], c.get("background", ()), c.get("single", ()), fix)
            mk, npar, ncell = rm.regions(*args)
            key = f"{c['name']}_{dim}d"
            out["para_" + key] = mk
            out["npar_" + key] = npar
            out["ncell_" + key] = ncell
            r, cc, v, nr, nc = rm.constraints(*args)
            out["cons_" + key] = np.column_stack([r, cc, v])
            out["cons_shape_" + key] = np.array([nr, nc])
            print(key, npar, ncell, "constraints", nr, "x", nc)
        # more than 50 regions: every region single, lowest background
        mc = Mesh(dim, m.nodes, m.cells, np.arange(m.cellCount(), dtype=np.int32), m.node_markers, m.boundaries,
                  m.boundary_markers, m.boundary_cells)
        rmc = R.RefMesh(mc)
        mk, npar, ncell = rmc.regions(True)
        out[f"para_many_{dim}d"] = mk
        out[f"npar_many_{dim}d"] = npar
        out[f"ncell_many_{dim}d"] = ncell
        r, cc, v, nr, nc = rmc.constraints(True)
        out[f"cons_many_{dim}d"] = np.column_stack([r, cc, v])
        out[f"cons_shape_many_{dim}d"] = np.array([nr, nc])
        print(f"many_{dim}d", npar, ncell, "constraints", nr, "x", nc)
    np.savez_compressed(OUT, cases=json.dumps(CASES), **out)


if __name__ == "__main__":
    main()
