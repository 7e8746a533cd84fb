"""Model -> per-cell resistivity mapping.

Restates ModellingBase::createMappedModel (core/src/modellingbase.cpp:401-497)
and
Mesh::prolongateEmptyCellsValues (core/src/mesh.cpp:2247-2316):
  * a model with one value per cell whose marker count differs is used as is;
  * otherwise cell c gets model[marker(c)];
  * marker -1 cells start empty and are filled with ``background`` when it
    is above -9e99, else iteratively from their face neighbours, weighted by
    the horizontal part of the shared facet normal plus 1e-6.
"""
from __future__ import annotations

import numpy as np

TOLERANCE = 1e-12
MARKER_FIXEDVALUE_REGION = -1000000  # core/src/gimli.h:241


def _neighbours(mesh):
    cells = mesh.cells
    nv = cells.shape[1]
    n = mesh.nodeCount()
    faces, owner = [], []
    for skip in range(nv):
        cols = [j for j in range(nv) if j != skip]
        faces.append(np.sort(cells[:, cols], axis=1))
        owner.append(np.arange(len(cells)))
    faces = np.concatenate(faces).astype(np.int64)
    owner = np.concatenate(owner)
    key = faces[:, 0]
    for j in range(1, faces.shape[1]):
        key = key * n + faces[:, j]
    order = np.argsort(key, kind="stable")
    key, owner, faces = key[order], owner[order], faces[order]
    pair = np.nonzero(key[1:] == key[:-1])[0]
    return owner[pair], owner[pair + 1], faces[pair]


def _facet_normals(mesh, faces):
    p = mesh.nodes[faces]
    if mesh.dim() == 2:
        t = p[:, 1] - p[:, 0]
        nrm = np.column_stack([t[:, 1], -t[:, 0], np.zeros(len(t))])
    else:
        nrm = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    return nrm / np.linalg.norm(nrm, axis=1)[:, None]


def prolongate_empty_cells(mesh, vals, background=-9e99):
    empty = np.nonzero(np.abs(vals) < TOLERANCE)[0]
    if len(empty) == 0:
        return vals
    if background > -9e99:
        vals[empty] = background
        return vals
    c1, c2, faces = _neighbours(mesh)
    XY = np.array([1.0, 1.0, 0.0])
    if mesh.dim() == 2:
        XY[1] = 0.0
    zw = np.linalg.norm(_facet_normals(mesh, faces) * XY, axis=1) + 1e-6
    while True:
        empty_mask = np.abs(vals) < TOLERANCE
        if not empty_mask.any():
            return vals
        vsum = np.zeros(len(vals))
        wsum = np.zeros(len(vals))
        for a, b in ((c1, c2), (c2, c1)):
            use = empty_mask[a] & ~empty_mask[b]
            np.add.at(vsum, a[use], vals[b[use]] * zw[use])
            np.add.at(wsum, a[use], zw[use])
        upd = empty_mask & (wsum > 1e-8)
        if not upd.any():
            raise ValueError("cannot prolongate values into empty cells")
        vals[upd] = vsum[upd] / wsum[upd]


def _marker_count(mesh):
    """Number of distinct non-negative cell markers (O(cells), cached for the
    mesh's current marker array)."""
    mk = mesh.cell_markers
    cached = getattr(mesh, "_marker_count_cache", None)
    if cached is not None and cached[0] is mk:
        return cached[1]
    pos = mk[mk >= 0]
    cnt = int(np.count_nonzero(np.bincount(pos))) if len(pos) else 0
    mesh._marker_count_cache = (mk, cnt)
    return cnt


def map_model(mesh, model, background=-9e99, fixed=None):
    """Per-cell resistivity for ``model`` (per cell or per marker); cells of
    fixed-value regions (marker MARKER_FIXEDVALUE_REGION - region) get
    ``fixed[region]`` after the prolongation (modellingbase.cpp:465-494)."""
    model = np.asarray(model, dtype=np.float64)
    mk = mesh.cell_markers
    C = mesh.cellCount()
    if len(model) == C and _marker_count(mesh) != len(model):
        return model.copy()
    att = np.zeros(C)
    pos = mk >= 0
    if np.any(mk[pos] >= len(model)):
        raise ValueError(f"marker >= model size ({mk.max()} >= {len(model)})")
    att[pos] = model[mk[pos]]
    if (~pos).all() and background != 0.0:
        raise ValueError("too many empty cells")
    if background != 0.0:
        prolongate_empty_cells(mesh, att, background)
    fx = mk <= MARKER_FIXEDVALUE_REGION
    if fx.any():
        if not fixed:
            raise ValueError("fixed-value region cells but no fixed values")
        regions = -(mk[fx].astype(np.int64) - MARKER_FIXEDVALUE_REGION)
        att[fx] = np.array([fixed[int(r)] for r in regions])
    return att
