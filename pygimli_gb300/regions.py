"""Region bookkeeping of a parameter mesh: the part of the reference's
``RegionManager`` that decides which cell carries which model parameter.

Restates core/src/regionManager.cpp: ``setMesh`` (617-689: one region per
distinct cell marker, ascending; more than 50 regions are all single),
``recountParaMarker_`` (760-766) with ``Region::countParameter`` (173-201:
a background region's cells get marker -1, or MARKER_FIXEDVALUE_REGION -
marker with a fixed value; a single region is one parameter; any other
region has one parameter per cell, in cell order), ``createParaDomain_``
(734-750: the cells of the regions that are not background), and pyGIMLi's
``MeshModelling.setDefaultBackground`` (pygimli/frameworks/modelling.py:
757-767: with several regions the lowest marker becomes background), and
the default first-order constraint matrix (``constraintMatrix``).  Other
constraint types, weights and transformation settings of regions belong to
the inversion framework and are not kept here.
"""
from __future__ import annotations

import numpy as np

from .mesh import Mesh

MARKER_FIXEDVALUE_REGION = -1000000  # core/src/gimli.h:241
TOLERANCE = 1e-12


class Region:
    """One region: its marker, its cells (ascending ids) and its flags."""

    def __init__(self, marker, cells, single=False):
        self.marker = int(marker)
        self.cells = np.asarray(cells, np.int64)
        self._background = False
        self._single = bool(single)
        # a region created single has constraint type 0 (no rows), any other
        # type 1 (Region::Region, core/src/regionManager.cpp:31-47)
        self.constraintType = 0 if single else 1
        self._fix = 0.0
        self.startParameter = 0
        self._count = 0

    def isBackground(self):
        return self._background

    def isSingle(self):
        return self._single

    def fixValue(self):
        return self._fix

    def parameterCount(self):
        return self._count

    def setBackground(self, b=True):
        self._background = bool(b)

    def setSingle(self, b=True):
        self._single = bool(b)

    def setFixValue(self, v):
        """A fixed region is background: its cells take the value, no parameter."""
        self._fix = float(v)
        self._background = True


class RegionManager:
    """Regions of a parameter mesh and the resulting parameter markers."""

    def __init__(self):
        self._regions = {}
        self._mesh = None
        self._markers = None

    def setMesh(self, mesh):
        self._mesh = mesh
        mk = np.asarray(mesh.cell_markers, np.int64)
        self._markers = mk.copy()  # the mesh copy's cell markers, renumbered by recount()
        uniq = np.unique(mk)
        single_only = len(uniq) > 50
        order = np.argsort(mk, kind="stable")
        bounds = np.searchsorted(mk[order], uniq)
        ends = np.append(bounds[1:], len(mk))
        self._regions = {int(m): Region(m, order[b:e], single_only) for m, b, e in zip(uniq, bounds, ends)}
        self.recount()

    def regionIdxs(self):
        return sorted(self._regions)

    def regionCount(self):
        return len(self._regions)

    def region(self, marker):
        if int(marker) not in self._regions:
            raise KeyError(f"no region with marker {marker}")
        return self._regions[int(marker)]

    def setRegionProperties(self, marker, background=None, single=None, fix=None):
        markers = self.regionIdxs() if marker == "*" else [marker]
        for m in markers:
            r = self.region(m)
            if background is not None:
                r.setBackground(background)
            if single is not None:
                r.setSingle(single)
            if fix is not None:
                r.setFixValue(fix)
        self.recount()

    def setDefaultBackground(self):
        """With several regions, the lowest marker is background."""
        ids = self.regionIdxs()
        if len(ids) > 1:
            self.setRegionProperties(ids[0], background=True)

    def recount(self):
        start = 0
        for m in self.regionIdxs():
            r = self._regions[m]
            r.startParameter = start
            c = r.cells
            if r.isBackground():
                if abs(r.fixValue()) > TOLERANCE:
                    sel = c[self._markers[c] >= -1]
                    self._markers[sel] = MARKER_FIXEDVALUE_REGION - m
                else:
                    self._markers[c] = -1
                r._count = 0
            elif r.isSingle():
                self._markers[c] = start
                r._count = 1
            else:
                self._markers[c] = start + np.arange(len(c))
                r._count = len(c)
            start += r._count

    def parameterCount(self):
        return int(sum(r.parameterCount() for r in self._regions.values()))

    def paraMarkers(self):
        """Cell markers of the parameter mesh: parameter index, -1 for
        background cells, MARKER_FIXEDVALUE_REGION - region for fixed ones."""
        return self._markers.astype(np.int32)

    def fixedValues(self):
        """{region marker: fixed value} of the fixed regions."""
        return {m: r.fixValue() for m, r in self._regions.items()
                if r.isBackground() and abs(r.fixValue()) > TOLERANCE}

    def paraDomain(self):
        """Mesh of the cells of non-background regions (Mesh::createMeshByCells,
        core/src/mesh.cpp:2008-2088: ascending cell ids, nodes renumbered in
        order of first use, the boundaries with a nonzero marker that lie on a
        kept cell, the cell data of the kept cells), with the parameter
        indices as cell markers."""
        mesh = self._mesh
        keep = np.sort(np.concatenate([r.cells for r in self._regions.values() if not r.isBackground()]
                                      or [np.zeros(0, np.int64)]))
        cells = mesh.cells[keep, :mesh.dim() + 1]
        used, first = np.unique(cells.ravel(), return_index=True)
        order = used[np.argsort(first, kind="stable")]
        remap = np.full(mesh.nodeCount(), -1, np.int64)
        remap[order] = np.arange(len(order))
        from .mesh import find_boundary_cells
        new_cells = remap[cells].astype(np.int32)
        b = mesh.boundaries[:, :mesh.dim()].astype(np.int64)
        sel = np.nonzero((mesh.boundary_markers != 0) & np.all(remap[b] >= 0, axis=1))[0]
        nb = remap[b[sel]].astype(np.int32)
        owner = find_boundary_cells(new_cells, nb, len(order))
        keep_b = owner >= 0
        pd = Mesh(mesh.dim(), mesh.nodes[order], new_cells, self._markers[keep].astype(np.int32),
                  mesh.node_markers[order], nb[keep_b], mesh.boundary_markers[sel][keep_b], owner[keep_b],
                  check=False)
        C = mesh.cellCount()
        pd._data = {k: v[keep].copy() for k, v in getattr(mesh, "_data", {}).items() if len(v) == C}
        return pd

    def constraintMatrix(self):
        """The default constraint matrix over the parameters
        (RegionManager::fillConstraints, core/src/regionManager.cpp:920-1040),
        as (rowptr, cols, vals, P) in CSR:

        * regions in marker order: a background (or fixed) region has no
          rows; a single region one row, +1 at its parameter, when it became
          single after its creation (constraint type 1), none when it was
          created single (type 0); every other region one first-order row
          per face shared by two of its cells, +1 and -1 at their parameters
          (Region::resize 132-159, Region::fillConstraints 371-396);
        * with more than 50 regions (all created single) the reference adds
          inter-region constraints between every pair of neighbouring
          regions (setMesh 617-689, fillConstraints 953-1040): per pair in
          marker order one row per shared face (one for the whole interface
          when both regions are single), +1 at the cell of the lower marker
          and -1 at the other; the rows of a pair with a background region
          are counted but stay empty (interRegionConstraintsCount 901-918);
        * no row at all: the identity (zeroth order, 929-938).

        Rows within a region follow the faces' sorted node ids (the
        reference: its boundary numbering), and the sign of a first-order row
        may differ from the reference's left / right cell; neither changes
        C^T C."""
        mesh = self._mesh
        P = self.parameterCount()
        a, b = interior_face_cells(mesh)
        reg = np.asarray(mesh.cell_markers, np.int64)
        para = self._markers
        counts, cols, vals = [], [], []
        for m in self.regionIdxs():
            r = self._regions[m]
            if r.isBackground():
                continue
            if r.isSingle():
                if r.constraintType == 1:
                    counts.append(np.ones(1, np.int64))
                    cols.append(np.array([r.startParameter], np.int64))
                    vals.append(np.ones(1))
                continue
            sel = (reg[a] == m) & (reg[b] == m)
            k = int(sel.sum())
            counts.append(np.full(k, 2, np.int64))
            cols.append(np.column_stack([para[a[sel]], para[b[sel]]]).ravel())
            vals.append(np.tile([1.0, -1.0], k))
        if len(self._regions) > 50:
            c, i, v = self._inter_region_rows(a, b, reg, para)
            counts.append(c)
            cols.append(i)
            vals.append(v)
        counts = np.concatenate(counts) if counts else np.zeros(0, np.int64)
        if len(counts) == 0:
            return np.arange(P + 1, dtype=np.int32), np.arange(P, dtype=np.int32), np.ones(P), P
        rowptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
        return rowptr, np.concatenate(cols).astype(np.int32), np.concatenate(vals).astype(np.float64), P

    def _inter_region_rows(self, a, b, reg, para):
        """(entries per row, cols, vals) of the inter-region rows between
        neighbouring regions, as constraintMatrix describes them."""
        ra, rb = reg[a], reg[b]
        sel = np.nonzero(ra != rb)[0]
        lo, hi = np.minimum(ra, rb)[sel], np.maximum(ra, rb)[sel]
        ca = np.where(ra < rb, a, b)[sel]
        cb = np.where(ra < rb, b, a)[sel]
        order = np.lexsort((np.arange(len(sel)), hi, lo))
        lo, hi, ca, cb = lo[order], hi[order], ca[order], cb[order]
        counts, cols, vals = [], [], []
        start = 0
        while start < len(lo):
            end = start
            while end < len(lo) and lo[end] == lo[start] and hi[end] == hi[start]:
                end += 1
            ra_, rb_ = self._regions[int(lo[start])], self._regions[int(hi[start])]
            n = 1 if (ra_.isSingle() and rb_.isSingle()) else end - start
            empty = ra_.isBackground() or rb_.isBackground()
            for q in range(start, start + n):
                counts.append(0 if empty else 2)
                if not empty:
                    cols += [para[ca[q]], para[cb[q]]]
                    vals += [1.0, -1.0]
            start = end
        return np.asarray(counts, np.int64), np.asarray(cols, np.int64), np.asarray(vals, np.float64)


def interior_face_cells(mesh):
    """Cell pairs (a < b) of the faces shared by two cells, in the order of
    the faces' sorted node ids."""
    cells = mesh.cells[:, :mesh.dim() + 1].astype(np.int64)
    nv = cells.shape[1]
    n = mesh.nodeCount()
    faces = np.concatenate([np.sort(cells[:, [j for j in range(nv) if j != skip]], axis=1) for skip in range(nv)])
    owner = np.tile(np.arange(len(cells)), nv)
    key = faces[:, 0]
    for j in range(1, faces.shape[1]):
        key = key * n + faces[:, j]
    order = np.lexsort((owner, key))
    key, owner = key[order], owner[order]
    pair = np.nonzero(key[1:] == key[:-1])[0]
    return owner[pair], owner[pair + 1]
