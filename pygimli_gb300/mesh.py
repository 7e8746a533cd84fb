"""Unstructured simplex mesh container and the synthetic mesh generators
used by the ERT forward operator.

The container mirrors the parts of ``GIMLI::Mesh`` that the DC forward
operator reads (core/src/mesh.h:183-217 node/cell/boundary creation,
core/src/mesh.h:345-351 accessors): node positions with node markers,
linear triangles (2-D) or tetrahedra (3-D) with cell markers, and boundary
facets with boundary markers and the adjacent ("left") cell.

Conventions follow the reference:
  * ``dim-1`` is the vertical axis; 2-D meshes use y as depth
    (core/src/bert/dcfemmodelling.cpp:859-867).
  * node marker -99 marks an electrode node (core/src/bert/bert.h:30).
  * boundary marker -1 is homogeneous Neumann (the surface), -2 is the
    mixed (Robin) far-field condition (core/src/gimli.h:235-236).

The generators restate the geometry of pyGIMLi's parameter meshes
(pygimli/meshtools/polytools.py:882 createParaMeshPLC: a para box of sensor
span plus a margin, a wide prolongation boundary with Neumann top and mixed
sides/bottom, electrode nodes with marker -99) with graded structured
triangulations instead of Triangle/TetGen, which are not part of this
project.  The 3-D box is split into tetrahedra like
pygimli/meshtools/mesh.py:448 refineHex2Tet (six tetrahedra per hexahedron
around the main diagonal).
"""
from __future__ import annotations

import os

import numpy as np

MARKER_NODE_ELECTRODE = -99
MARKER_BOUND_HOMOGEN_NEUMANN = -1
MARKER_BOUND_MIXED = -2
MARKER_BOUND_HOMOGEN_DIRICHLET = -3


class Mesh:
    """Simplex mesh: triangles (2-D) or tetrahedra (3-D), linear (P1) or
    quadratic (P2: Triangle6 / Tetrahedron10 with edge-midpoint nodes)."""

    def __init__(self, dim, nodes, cells, cell_markers=None, node_markers=None,
                 boundaries=None, boundary_markers=None, boundary_cells=None, check=True):
        """``check=False`` skips the degenerate-cell test (for refinements of
        a checked mesh, whose children are never degenerate)."""
        self.dim_ = int(dim)
        nodes = np.asarray(nodes, dtype=np.float64)
        if nodes.shape[1] == 2:
            nodes = np.column_stack([nodes, np.zeros(len(nodes))])
        self.nodes = np.ascontiguousarray(nodes)
        self.cells = np.ascontiguousarray(np.asarray(cells, dtype=np.int32))
        nv1 = self.dim_ + 1
        nv2 = 6 if self.dim_ == 2 else 10
        if self.cells.ndim != 2 or self.cells.shape[1] not in (nv1, nv2):
            raise ValueError(f"cells must be (C, {nv1}) or (C, {nv2}) for a {dim}-D simplex mesh")
        self.order = 1 if self.cells.shape[1] == nv1 else 2
        nvb = self.dim_ if self.order == 1 else (3 if self.dim_ == 2 else 6)
        C = len(self.cells)
        self.cell_markers = (np.arange(C, dtype=np.int32) if cell_markers is None
                             else np.ascontiguousarray(np.asarray(cell_markers, dtype=np.int32)))
        self.node_markers = (np.zeros(len(self.nodes), np.int32) if node_markers is None
                             else np.ascontiguousarray(np.asarray(node_markers, dtype=np.int32)))
        if boundaries is None:
            boundaries = np.zeros((0, nvb), np.int32)
            boundary_markers = np.zeros(0, np.int32)
        self.boundaries = np.ascontiguousarray(np.asarray(boundaries, dtype=np.int32).reshape(-1, nvb))
        self.boundary_markers = np.ascontiguousarray(np.asarray(boundary_markers, dtype=np.int32))
        if boundary_cells is None:
            boundary_cells = find_boundary_cells(self.cells[:, :nv1], self.boundaries[:, :self.dim_],
                                                 len(self.nodes))
        self.boundary_cells = np.ascontiguousarray(np.asarray(boundary_cells, dtype=np.int32))
        # left / right cell of each boundary as the binary mesh format stores
        # them (-1: none or not known); boundary_cells is the adjacent cell
        self.boundary_left_cells = self.boundary_cells.copy()
        self.boundary_right_cells = np.full(len(self.boundaries), -1, np.int32)
        self.geometry = False
        self._data = {}
        if check and np.any(self._signed_sizes() == 0):
            raise ValueError("degenerate cell in mesh")

    # -- reference-style accessors (core/src/mesh.h:331-351) --------------
    def dim(self):
        return self.dim_

    def dimension(self):
        return self.dim_

    def nodeCount(self):
        return len(self.nodes)

    def cellCount(self):
        return len(self.cells)

    def boundaryCount(self):
        return len(self.boundaries)

    def cellMarkers(self):
        return self.cell_markers.copy()

    def setCellMarkers(self, markers):
        m = np.asarray(markers, dtype=np.int32)
        if m.shape != (self.cellCount(),):
            raise ValueError("marker count does not match the cell count")
        self.cell_markers = np.ascontiguousarray(m)

    def positions(self):
        return self.nodes.copy()

    def findNodesIdxByMarker(self, marker):
        return np.nonzero(self.node_markers == marker)[0]

    def _signed_sizes(self):
        p = self.nodes[self.cells[:, :self.dim_ + 1]]
        if self.dim_ == 2:
            a = p[:, 1, :2] - p[:, 0, :2]
            b = p[:, 2, :2] - p[:, 0, :2]
            return a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0]
        a = p[:, 1] - p[:, 0]
        b = p[:, 2] - p[:, 0]
        c = p[:, 3] - p[:, 0]
        return np.einsum("ij,ij->i", a, np.cross(b, c))

    def createP2(self):
        """Quadratic mesh, see create_p2."""
        return create_p2(self)

    def createH2(self):
        """Uniformly refined mesh, see create_h2."""
        return create_h2(self)

    def cellSizes(self):
        """Cell areas (2-D) or volumes (3-D), positive."""
        p = self.nodes[self.cells[:, :self.dim_ + 1]]
        if self.dim_ == 2:
            a = p[:, 1, :2] - p[:, 0, :2]
            b = p[:, 2, :2] - p[:, 0, :2]
            return 0.5 * np.abs(a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0])
        a = p[:, 1] - p[:, 0]
        b = p[:, 2] - p[:, 0]
        c = p[:, 3] - p[:, 0]
        return np.abs(np.einsum("ij,ij->i", a, np.cross(b, c))) / 6.0

    def cellCenters(self):
        return self.nodes[self.cells[:, :self.dim_ + 1]].mean(axis=1)

    # -- data map (core/src/mesh.h:603-640) ----------------------------------
    def addData(self, name, values):
        self._data[str(name)] = np.asarray(values, np.float64).copy()

    def data(self, name):
        return self._data[name].copy()

    def haveData(self, name):
        return name in self._data

    def dataMap(self):
        return {k: v.copy() for k, v in self._data.items()}

    def __setitem__(self, name, values):
        self.addData(name, values)

    def __getitem__(self, name):
        return self.data(name)

    # -- files ------------------------------------------------------------------
    def save(self, path):
        """Binary mesh file (the reference's Mesh::save, format v3, '.bms'
        appended when missing), or a numpy archive for a '.npz' name.
        Returns the file name written."""
        path = os.fspath(path)
        if path.endswith(".npz"):
            np.savez_compressed(path, dim=self.dim_, nodes=self.nodes, cells=self.cells,
                                cell_markers=self.cell_markers, node_markers=self.node_markers,
                                boundaries=self.boundaries, boundary_markers=self.boundary_markers,
                                boundary_cells=self.boundary_cells)
            return path
        from .fileio import write_bms
        return write_bms(path, self.dim_, self.nodes, self.node_markers, self.cells, self.cell_markers,
                         self.boundaries, self.boundary_markers, self.boundary_left_cells, self.boundary_right_cells,
                         self._data, self.geometry)

    def saveBinaryV2(self, path):
        """Binary mesh file, format v3 (Mesh::saveBinaryV2)."""
        return self.save(os.fspath(path) if os.fspath(path).endswith(".bms") else os.fspath(path) + ".bms")

    def saveBinary(self, path):
        """The first binary mesh format (Mesh::saveBinary); no data map."""
        from .fileio import write_bms_v1
        return write_bms_v1(os.fspath(path), self.dim_, self.nodes, self.node_markers, self.cells, self.cell_markers,
                            self.boundaries, self.boundary_markers, self.boundary_left_cells,
                            self.boundary_right_cells, self.geometry)

    @staticmethod
    def load(path):
        """Mesh from a binary mesh file (Mesh::loadBinaryV2, versions 2 and
        3, else the first format of Mesh::loadBinary) or a numpy archive
        written by ``save``."""
        path = os.fspath(path)
        if path.endswith(".vtk"):
            return Mesh.importVTK(path)
        if path.endswith(".npz"):
            z = np.load(path)
            return Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"],
                        z["boundaries"], z["boundary_markers"], z["boundary_cells"])
        from .fileio import read_bms
        r = read_bms(path)
        if isinstance(r["cells"], list) or isinstance(r["boundaries"], list):
            raise ValueError("mixed cell or boundary types: only simplex meshes are supported")
        bnd = r["boundaries"]
        if len(bnd) == 0:
            nv = r["cells"].shape[1] if len(r["cells"]) else r["dim"] + 1
            nvb = r["dim"] if nv == r["dim"] + 1 else (3 if r["dim"] == 2 else 6)
            bnd = np.zeros((0, nvb), np.int32)
        # adjacent cell: left, else right, else searched (the reference's
        # mixed-boundary assembly, core/src/bert/dcfemmodelling.cpp:258-260)
        adj = np.where(r["left"] >= 0, r["left"], r["right"]).astype(np.int32)
        if np.any(adj < 0):
            nv1 = r["dim"] + 1
            found = find_boundary_cells(np.asarray(r["cells"])[:, :nv1], bnd[:, :r["dim"]], len(r["nodes"]))
            adj = np.where(adj >= 0, adj, found).astype(np.int32)
        m = Mesh(r["dim"], r["nodes"], r["cells"], r["cell_markers"], r["node_markers"], bnd,
                 r["boundary_markers"], adj)
        m.boundary_left_cells = np.ascontiguousarray(r["left"], np.int32)
        m.boundary_right_cells = np.ascontiguousarray(r["right"], np.int32)
        m.geometry = r["geometry"]
        m._data = r["data"]
        return m

    @staticmethod
    def importVTK(path):
        """Mesh from a legacy ASCII VTK unstructured grid (Mesh::importVTK):
        nodes, cells, the SCALARS arrays as data and 'Marker' as cell
        markers; no boundaries and no node markers (as the reference)."""
        from .fileio import read_vtk
        r = read_vtk(os.fspath(path))
        m = Mesh(r["dim"], r["nodes"], r["cells"], r["cell_markers"], check=False)
        m._data = r["data"]
        return m

    def exportVTK(self, fbody, writeCells=True):
        """Legacy ASCII VTK file (Mesh::exportVTK): nodes, cells with types,
        the data map entries of cell (node) length as cell (point) scalars
        plus the cell markers as 'Marker'.  Returns the file name."""
        from .fileio import write_vtk
        return write_vtk(os.fspath(fbody), self.dim_, self.nodes, self.cells, self.cell_markers, self.boundaries,
                         self.boundary_markers, self._data, writeCells)

    def __repr__(self):
        return (f"Mesh(dim={self.dim_}, order={self.order}, nodes={self.nodeCount()}, "
                f"cells={self.cellCount()}, boundaries={self.boundaryCount()})")


# Tetrahedron10 node order (Zienkiewicz): vertices, then edges 01 02 03 12 23 31
_TET10_EDGES = ((0, 1), (0, 2), (0, 3), (1, 2), (2, 3), (3, 1))
# Triangle6: vertices, then edges 01 12 20
_TRI6_EDGES = ((0, 1), (1, 2), (2, 0))


def _marker_mid(m0, m1):
    """Marker of an edge-midpoint node (core/src/mesh.cpp:1293-1299)."""
    if m0 == -99 and m1 == -99:
        return -1
    if m0 == -99:
        return m1
    if m1 == -99:
        return m0
    return m1 if m0 == m1 else 0


def _edge_midpoints(mesh, pairs_c, pairs_b):
    """Node ids of the midpoints of the edge pairs, created in order of first
    use (Mesh::createRefinementNode_, core/src/mesh.cpp:1301-1313): new
    nodes, their markers (markerT) and the ids of the cell / boundary pairs."""
    n0 = mesh.nodeCount()
    pairs = np.concatenate([pairs_c, pairs_b])
    key = np.minimum(pairs[:, 0], pairs[:, 1]) * n0 + np.maximum(pairs[:, 0], pairs[:, 1])
    uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
    order = np.argsort(first, kind="stable")
    rank = np.empty(len(uniq), np.int64)
    rank[order] = np.arange(len(uniq))
    mid_id = n0 + rank[inv]
    ea = pairs[first[order], 0]
    eb = pairs[first[order], 1]
    mids = 0.5 * (mesh.nodes[ea] + mesh.nodes[eb])
    nm = mesh.node_markers
    mid_markers = np.array([_marker_mid(int(nm[a]), int(nm[b])) for a, b in zip(ea, eb)], np.int32)
    return mids, mid_markers, mid_id[:len(pairs_c)], mid_id[len(pairs_c):]


# H2 children in terms of the Tetrahedron10 nodes (core/src/mesh.cpp:1399-1406)
_TET_H2 = ((4, 6, 5, 0), (4, 5, 6, 9), (7, 9, 4, 1), (7, 4, 9, 5),
           (8, 7, 5, 2), (8, 5, 7, 9), (6, 9, 8, 3), (6, 8, 9, 5))
# ... and of the Triangle6 nodes (mesh.cpp:1357-1362)
_TRI_H2 = ((0, 3, 5), (1, 4, 3), (2, 5, 4), (3, 4, 5))


def create_h2(mesh):
    """Uniform refinement (every cell split into 4 triangles / 8 tetrahedra)
    with the node, cell and boundary numbering of Mesh::createH2
    (core/src/mesh.cpp:1278-1283, createRefined_): children follow their
    parent in cell order and inherit its marker; boundary edges / faces are
    split into 2 / 4 with the parent's marker.  pyGIMLi uses this as the
    forward mesh of a parameter mesh (pygimli/frameworks/modelling.py:586,
    682-699)."""
    if mesh.order != 1:
        raise ValueError("H2 refinement of a quadratic mesh is not supported")
    edges = _TET10_EDGES if mesh.dim() == 3 else _TRI6_EDGES
    cells = mesh.cells.astype(np.int64)
    C = len(cells)
    pairs_c = np.stack([cells[:, [a for a, _ in edges]], cells[:, [b for _, b in edges]]], axis=2).reshape(-1, 2)
    bnd = mesh.boundaries.astype(np.int64)
    bedges = ((0, 1), (1, 2), (2, 0)) if mesh.dim() == 3 else ((0, 1),)
    pairs_b = np.stack([bnd[:, [a for a, _ in bedges]], bnd[:, [b for _, b in bedges]]], axis=2).reshape(-1, 2)
    mids, mid_markers, cm, bm = _edge_midpoints(mesh, pairs_c, pairs_b)
    full = np.concatenate([cells, cm.reshape(C, len(edges))], axis=1)
    children = _TET_H2 if mesh.dim() == 3 else _TRI_H2
    cells2 = full[:, np.array(children)].reshape(-1, mesh.dim() + 1)
    markers2 = np.repeat(mesh.cell_markers, len(children))
    bfull = np.concatenate([bnd, bm.reshape(len(bnd), len(bedges))], axis=1)
    if mesh.dim() == 3:
        bnd2 = bfull[:, np.array(_TRI_H2)].reshape(-1, 3)
        bmk = np.repeat(mesh.boundary_markers, 4)
    else:
        bnd2 = bfull[:, np.array(((0, 2), (2, 1)))].reshape(-1, 2)
        bmk = np.repeat(mesh.boundary_markers, 2)
    nodes = np.concatenate([mesh.nodes, mids])
    node_markers = np.concatenate([mesh.node_markers, mid_markers])
    return Mesh(mesh.dim(), nodes, cells2.astype(np.int32), markers2, node_markers, bnd2.astype(np.int32), bmk,
                check=False)


def create_p2(mesh):
    """Quadratic (P2) mesh with the node numbering of Mesh::createP2
    (core/src/mesh.cpp:1284-1288, createRefined_ 1315-1600): the P1 nodes keep
    their ids; a midpoint node is created for every edge at its first use,
    walking the cells in order and each cell's edges in Tetrahedron10
    (Zienkiewicz) / Triangle6 order, then the boundaries.  Every cell keeps
    its marker (createRefined_ maps the parent marker onto the new cells);
    boundary markers are kept."""
    if mesh.order != 1:
        raise ValueError("mesh is already quadratic")
    edges = _TET10_EDGES if mesh.dim() == 3 else _TRI6_EDGES
    cells = mesh.cells.astype(np.int64)
    C = len(cells)
    # candidate midpoints in creation order: cells (edge order), then boundaries
    pairs_c = np.stack([cells[:, [a for a, _ in edges]], cells[:, [b for _, b in edges]]], axis=2).reshape(-1, 2)
    bnd = mesh.boundaries.astype(np.int64)
    bedges = ((0, 1), (1, 2), (2, 0)) if mesh.dim() == 3 else ((0, 1),)
    pairs_b = np.stack([bnd[:, [a for a, _ in bedges]], bnd[:, [b for _, b in bedges]]], axis=2).reshape(-1, 2)
    mids, mid_markers, cm, bm = _edge_midpoints(mesh, pairs_c, pairs_b)
    nodes = np.concatenate([mesh.nodes, mids])
    node_markers = np.concatenate([mesh.node_markers, mid_markers])
    cells2 = np.concatenate([cells, cm.reshape(C, len(edges))], axis=1).astype(np.int32)
    bnd2 = np.concatenate([bnd, bm.reshape(len(bnd), len(bedges))], axis=1).astype(np.int32)
    return Mesh(mesh.dim(), nodes, cells2, mesh.cell_markers.copy(), node_markers, bnd2,
                mesh.boundary_markers.copy(), mesh.boundary_cells.copy(), check=False)


def _facet_keys(facets, n_nodes):
    f = np.sort(np.asarray(facets, dtype=np.int64), axis=1)
    key = f[:, 0]
    for j in range(1, f.shape[1]):
        key = key * n_nodes + f[:, j]
    return key


def find_boundary_cells(cells, boundaries, n_nodes):
    """Cell adjacent to each boundary facet (the reference's leftCell,
    core/src/bert/dcfemmodelling.cpp:251-255).  -1 where none is found."""
    if len(boundaries) == 0:
        return np.zeros(0, np.int32)
    nv = cells.shape[1]
    faces = []
    owner = []
    for skip in range(nv):
        cols = [j for j in range(nv) if j != skip]
        faces.append(cells[:, cols])
        owner.append(np.arange(len(cells)))
    faces = np.concatenate(faces)
    owner = np.concatenate(owner)
    fk = _facet_keys(faces, n_nodes)
    order = np.argsort(fk, kind="stable")
    fk = fk[order]
    owner = owner[order]
    bk = _facet_keys(boundaries, n_nodes)
    pos = np.searchsorted(fk, bk)
    pos = np.minimum(pos, len(fk) - 1)
    ok = fk[pos] == bk
    out = np.where(ok, owner[pos], -1).astype(np.int32)
    return out


def _graded_axis(fine_lo, fine_hi, h, outer_lo, outer_hi, growth, must_include=()):
    """Node coordinates: uniform spacing ``h`` on [fine_lo, fine_hi] (hitting
    every value of ``must_include``), geometric growth towards the outer
    bounds."""
    n = int(round((fine_hi - fine_lo) / h))
    core = fine_lo + h * np.arange(n + 1)
    core[-1] = fine_hi
    for v in must_include:
        if np.min(np.abs(core - v)) > 1e-9 * max(1.0, abs(v)):
            raise ValueError(f"grid spacing {h} does not hit required coordinate {v}")
    left = []
    x, d = fine_lo, h
    while x > outer_lo + 1e-9:
        d *= growth
        x = max(x - d, outer_lo)
        if x - outer_lo < 0.5 * d:
            x = outer_lo
        left.append(x)
    right = []
    x, d = fine_hi, h
    while x < outer_hi - 1e-9:
        d *= growth
        x = min(x + d, outer_hi)
        if outer_hi - x < 0.5 * d:
            x = outer_hi
        right.append(x)
    return np.concatenate([np.array(left[::-1]), core, np.array(right)])


def create_para_mesh_2d(sensors_x, para_dx=0.25, para_depth=10.0, para_boundary=2.0,
                        boundary=-1.0, depth_growth=1.3, side_growth=1.6):
    """2-D (x, y=depth) parameter mesh for a surface electrode line.

    Geometry follows createParaMeshPLC (pygimli/meshtools/polytools.py:882):
    the para box spans the sensors plus ``para_boundary`` sensor spacings and
    reaches ``para_depth``; the prolongation boundary is ``4 x`` the para
    width on each side and below when ``boundary < 0``.  Surface nodes are
    placed every ``para_dx`` sensor spacing; electrode nodes carry marker -99.
    The surface (y=0) is Neumann (-1), sides and bottom are mixed (-2).
    Every cell gets its own marker (cell index), so the model is per cell.
    """
    xs = np.sort(np.asarray(sensors_x, dtype=np.float64))
    spacing = float(np.min(np.diff(xs)))
    h = spacing * para_dx
    x0 = xs[0] - para_boundary * spacing
    x1 = xs[-1] + para_boundary * spacing
    width = x1 - x0
    bnd = 4.0 * width if boundary < 0 else boundary * width
    xg = _graded_axis(x0, x1, h, x0 - bnd, x1 + bnd, side_growth, must_include=xs)
    # depth axis: geometric refinement from h at the surface to the para depth
    ys = [0.0]
    d = h
    while ys[-1] > -para_depth + 1e-9:
        nxt = ys[-1] - d
        if nxt < -para_depth + 0.5 * d:
            nxt = -para_depth
        ys.append(nxt)
        d *= depth_growth
    yb = -para_depth - bnd
    while ys[-1] > yb + 1e-9:
        d *= side_growth
        nxt = ys[-1] - d
        if nxt - yb < 0.5 * d:
            nxt = yb
        ys.append(max(nxt, yb))
    yg = np.array(ys)
    return _structured_tri_mesh(xg, yg, xs)


def _structured_tri_mesh(xg, yg, electrode_x):
    nx, ny = len(xg), len(yg)
    X, Y = np.meshgrid(xg, yg, indexing="ij")
    nodes = np.column_stack([X.ravel(), Y.ravel(), np.zeros(nx * ny)])

    def nid(i, j):
        return i * ny + j

    I, J = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), indexing="ij")
    I = I.ravel()
    J = J.ravel()
    a = nid(I, J)
    b = nid(I + 1, J)
    c = nid(I + 1, J + 1)
    d = nid(I, J + 1)
    alt = ((I + J) % 2) == 0
    t1 = np.where(alt[:, None], np.column_stack([a, b, c]), np.column_stack([a, b, d]))
    t2 = np.where(alt[:, None], np.column_stack([a, c, d]), np.column_stack([b, c, d]))
    cells = np.empty((2 * len(a), 3), np.int64)
    cells[0::2] = t1
    cells[1::2] = t2
    node_markers = np.zeros(nx * ny, np.int32)
    for ex in electrode_x:
        i = int(np.argmin(np.abs(xg - ex)))
        node_markers[nid(i, 0)] = MARKER_NODE_ELECTRODE
    bnds, bm = [], []
    for i in range(nx - 1):  # top (y = 0): Neumann
        bnds.append((nid(i, 0), nid(i + 1, 0)))
        bm.append(MARKER_BOUND_HOMOGEN_NEUMANN)
    for i in range(nx - 1):  # bottom
        bnds.append((nid(i, ny - 1), nid(i + 1, ny - 1)))
        bm.append(MARKER_BOUND_MIXED)
    for j in range(ny - 1):  # left / right
        bnds.append((nid(0, j), nid(0, j + 1)))
        bm.append(MARKER_BOUND_MIXED)
        bnds.append((nid(nx - 1, j), nid(nx - 1, j + 1)))
        bm.append(MARKER_BOUND_MIXED)
    return Mesh(2, nodes, cells.astype(np.int32), None, node_markers,
                np.array(bnds, np.int32), np.array(bm, np.int32))


# six tetrahedra per hexahedron around the diagonal v0-v6 (Kuhn split);
# hexahedron vertex order: v0=(0,0,0) v1=(1,0,0) v2=(1,1,0) v3=(0,1,0)
# v4=(0,0,1) v5=(1,0,1) v6=(1,1,1) v7=(0,1,1)
_KUHN = np.array([[0, 1, 2, 6], [0, 2, 3, 6], [0, 3, 7, 6],
                  [0, 7, 4, 6], [0, 4, 5, 6], [0, 5, 1, 6]], np.int64)


def create_box_mesh_3d(electrodes_xy, h=4.0 / 3.0, para_margin=(6, 5), para_depth=20.0,
                       outer=500.0, growth=1.45, depth_h=None, depth_growth=1.1):
    """3-D tetrahedral mesh of a para box padded to +-``outer`` m.

    Surface electrodes at ``electrodes_xy`` (z=0, marker -99).  The para box
    spans the electrode extent plus ``para_margin`` (x, y) cells of size
    ``h`` (which must hit every electrode coordinate) and reaches
    ``para_depth``; outside it the spacing grows geometrically to the outer
    boundary.  The top face is Neumann (-1), the other five faces are mixed
    (-2).  Every hexahedron is split into six tetrahedra (refineHex2Tet,
    pygimli/meshtools/mesh.py:448).  Every cell gets its own marker.
    """
    e = np.asarray(electrodes_xy, dtype=np.float64)
    ex = np.unique(e[:, 0])
    ey = np.unique(e[:, 1])
    mx, my = para_margin[0] * h, para_margin[1] * h
    xg = _graded_axis(ex[0] - mx, ex[-1] + mx, h, -outer, outer, growth, must_include=ex)
    yg = _graded_axis(ey[0] - my, ey[-1] + my, h, -outer, outer, growth, must_include=ey)
    dh = h if depth_h is None else depth_h
    zs = [0.0]
    d = dh
    while zs[-1] > -para_depth + 1e-9:
        nxt = zs[-1] - d
        if nxt < -para_depth + 0.5 * d:
            nxt = -para_depth
        zs.append(nxt)
        d *= depth_growth
    while zs[-1] > -outer + 1e-9:
        d *= growth
        nxt = zs[-1] - d
        if nxt + outer < 0.5 * d:
            nxt = -outer
        zs.append(max(nxt, -outer))
    zg = np.array(zs)
    return _structured_tet_mesh(xg, yg, zg, e)


def _structured_tet_mesh(xg, yg, zg, electrodes_xy):
    nx, ny, nz = len(xg), len(yg), len(zg)
    X, Y, Z = np.meshgrid(xg, yg, zg, indexing="ij")
    nodes = np.column_stack([X.ravel(), Y.ravel(), Z.ravel()])

    def nid(i, j, k):
        return (i * ny + j) * nz + k

    I, J, K = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1), np.arange(nz - 1), indexing="ij")
    I, J, K = I.ravel(), J.ravel(), K.ravel()
    # z index grows downward (z decreasing); vertex order is a right-handed
    # hexahedron up to orientation, fixed afterwards by Mesh._fix_orientation
    hv = np.column_stack([nid(I, J, K), nid(I + 1, J, K), nid(I + 1, J + 1, K), nid(I, J + 1, K),
                          nid(I, J, K + 1), nid(I + 1, J, K + 1), nid(I + 1, J + 1, K + 1),
                          nid(I, J + 1, K + 1)])
    cells = hv[:, _KUHN].reshape(-1, 4)
    node_markers = np.zeros(len(nodes), np.int32)
    for (x, y) in electrodes_xy:
        i = int(np.argmin(np.abs(xg - x)))
        j = int(np.argmin(np.abs(yg - y)))
        node_markers[nid(i, j, 0)] = MARKER_NODE_ELECTRODE
    # boundary faces: every hexahedron face on the box surface split like
    # the Kuhn tetrahedra split it (each face diagonal passes through the
    # face vertex with the smallest local index sum on the v0-v6 diagonal)
    faces, fm = [], []
    all_faces = np.concatenate([cells[:, [0, 1, 2]], cells[:, [0, 1, 3]],
                                cells[:, [0, 2, 3]], cells[:, [1, 2, 3]]])
    key = _facet_keys(all_faces, len(nodes))
    uniq, counts = np.unique(key, return_counts=True)
    outer_keys = uniq[counts == 1]
    sel = np.isin(key, outer_keys)
    bf = all_faces[sel]
    c = nodes[bf].mean(axis=1)
    top = np.isclose(c[:, 2], zg[0])
    fm = np.where(top, MARKER_BOUND_HOMOGEN_NEUMANN, MARKER_BOUND_MIXED).astype(np.int32)
    return Mesh(3, nodes, cells.astype(np.int32), None, node_markers, bf.astype(np.int32), fm)
