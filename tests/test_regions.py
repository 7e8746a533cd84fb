"""Region bookkeeping (regions.py) against the reference's own
RegionManager (core/src/regionManager.cpp) on the fixtures of
tests/golden/make_regions_golden.py: renumbered cell markers (parameter
indices, -1 background, MARKER_FIXEDVALUE_REGION - region for fixed
regions), parameter count, para-domain size and the constraint matrix
(RegionManager::fillConstraints: the same rows up to their order and sign,
the same row and column counts)."""
from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

from pygimli_gb300.mesh import Mesh
from pygimli_gb300.modelmap import map_model
from pygimli_gb300.regions import MARKER_FIXEDVALUE_REGION, RegionManager

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
from make_regions_golden import region_mesh  # noqa: E402

Z = np.load(os.path.join(GOLDEN, "regions.npz"))
CASES = json.loads(str(Z["cases"]))


def _rm(mesh, c):
    rm = RegionManager()
    rm.setMesh(mesh)
    if c.get("default_background"):
        rm.setDefaultBackground()
    for m in c.get("background", ()):
        rm.setRegionProperties(m, background=True)
    for m in c.get("single", ()):
        rm.setRegionProperties(m, single=True)
    for m, v in c.get("fix", {}).items():
        rm.setRegionProperties(int(m), fix=v)
    return rm


@pytest.mark.parametrize("dim", (2, 3))
@pytest.mark.parametrize("c", CASES, ids=[c["name"] for c in CASES])
def test_regions_match_reference(dim, c):
    m = region_mesh(dim)
    assert np.array_equal(m.cell_markers, Z[f"markers_{dim}d"])
    rm = _rm(m, c)
    key = f"{c['name']}_{dim}d"
    assert np.array_equal(rm.paraMarkers(), Z["para_" + key])
    assert rm.parameterCount() == int(Z["npar_" + key])
    assert rm.paraDomain().cellCount() == int(Z["ncell_" + key])


@pytest.mark.parametrize("dim", (2, 3))
def test_many_regions_are_single(dim):
    m = region_mesh(dim)
    mc = Mesh(dim, m.nodes, m.cells, np.arange(m.cellCount(), dtype=np.int32), m.node_markers, m.boundaries,
              m.boundary_markers, m.boundary_cells)
    rm = RegionManager()
    rm.setMesh(mc)
    rm.setDefaultBackground()
    assert all(rm.region(i).isSingle() for i in rm.regionIdxs())
    assert np.array_equal(rm.paraMarkers(), Z[f"para_many_{dim}d"])
    assert rm.parameterCount() == int(Z[f"npar_many_{dim}d"])


def test_mapping_with_background_and_fixed_region():
    """Background cells are filled from their neighbours, fixed-region cells
    take the region's value (createMappedModel, modellingbase.cpp:401-497)."""
    m = region_mesh(2)
    rm = _rm(m, {"default_background": True, "fix": {"3": 50.0}})
    para = Mesh(2, m.nodes, m.cells, rm.paraMarkers(), m.node_markers, m.boundaries, m.boundary_markers,
                m.boundary_cells)
    model = np.linspace(10.0, 20.0, rm.parameterCount())
    att = map_model(para, model, fixed=rm.fixedValues())
    mk = rm.paraMarkers()
    assert np.array_equal(att[mk >= 0], model[mk[mk >= 0]])
    assert np.all(att[mk == MARKER_FIXEDVALUE_REGION - 3] == 50.0)
    bg = mk == -1
    assert bg.any() and np.all((att[bg] >= 10.0 - 1e-9) & (att[bg] <= 20.0 + 1e-9))  # weighted means
    pd = rm.paraDomain()
    assert pd.cellCount() == int((mk >= 0).sum())
    assert np.array_equal(np.unique(pd.cell_markers), np.arange(rm.parameterCount()))


def test_para_domain_boundaries_and_data():
    """The para domain keeps the marked boundaries that lie on kept cells
    and the cell data of the kept cells (createMeshByCells)."""
    m = region_mesh(2)
    m["res"] = np.arange(m.cellCount(), dtype=float)
    rm = RegionManager()
    rm.setMesh(m)
    rm.setDefaultBackground()
    pd = rm.paraDomain()
    keep = np.nonzero(m.cell_markers != 1)[0]
    assert np.array_equal(pd["res"], keep.astype(float))
    assert pd.boundaryCount() > 0 and np.all(pd.boundary_markers != 0) and np.all(pd.boundary_cells >= 0)
    # every kept boundary is a face of its cell
    for bnd, c in zip(pd.boundaries, pd.boundary_cells):
        assert set(bnd.tolist()) <= set(pd.cells[c].tolist())


def _normalized_rows(rowptr, cols, vals):
    """Rows as sorted (column, value) tuples, each scaled to +1 at its lowest
    column: row order and sign leave C^T C unchanged."""
    out = []
    for i in range(len(rowptr) - 1):
        c, v = cols[rowptr[i]:rowptr[i + 1]], vals[rowptr[i]:rowptr[i + 1]]
        o = np.argsort(c)
        c, v = c[o], v[o]
        if len(v):
            v = v * np.sign(v[0])
        out.append(tuple(zip(c.tolist(), v.tolist())))
    return sorted(out)


def _reference_rows(key):
    t = Z["cons_" + key]
    nr, nc = (int(x) for x in Z["cons_shape_" + key])
    r = t[:, 0].astype(np.int64)
    o = np.lexsort((t[:, 1], r))
    rowptr = np.searchsorted(r[o], np.arange(nr + 1))
    return _normalized_rows(rowptr, t[o, 1].astype(np.int64), t[o, 2]), nr, nc


@pytest.mark.parametrize("dim", (2, 3))
@pytest.mark.parametrize("c", CASES + [{"name": "many"}], ids=[c["name"] for c in CASES] + ["many"])
def test_constraints_match_reference(dim, c):
    m = region_mesh(dim)
    if c["name"] == "many":  # every cell its own region: all single, inter-region rows
        m = Mesh(dim, m.nodes, m.cells, np.arange(m.cellCount(), dtype=np.int32), m.node_markers, m.boundaries,
                 m.boundary_markers, m.boundary_cells)
        c = {"name": "many", "default_background": True}
    rm = _rm(m, c)
    rowptr, cols, vals, P = rm.constraintMatrix()
    ref, nr, nc = _reference_rows(f"{c['name']}_{dim}d")
    assert (len(rowptr) - 1, P) == (nr, nc)
    assert _normalized_rows(rowptr, cols, vals) == ref
