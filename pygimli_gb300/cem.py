"""Electrodes of the total-potential operator: node electrodes, the complete
electrode model (CEM) and bypass electrodes, and the constant extension of
the system matrix they need.

pyGIMLi's ``ERTModelling(sr=False)`` (``DCMultiElectrodeModelling``) finds
three kinds of electrodes on the mesh (core/src/bert/dcfemmodelling.cpp:
790-1030):

* CEM electrodes: boundaries with marker ``-10000 - i`` (or cells with such
  a marker) form electrode ``i``; marker ``-9999`` marks a passive
  conductor (a "passive body");
* bypass electrodes: nodes with marker ``-10000 - i`` when no boundary or
  cell carries that marker; consecutive nodes of one marker are joined by
  bypass resistors (1e-6 Ohm by default) and the electrode sits on the
  first of them;
* node electrodes: nodes with marker -99 within 1 cm of a sensor.

Sensors are matched in that order.  With at least one CEM electrode or
passive body, every electrode and passive body gets one extra unknown, its
potential: the matrix grows by those rows and columns
(assembleCompleteElectrodeModel_, dcfemmodelling.cpp:315-414), the current
of an electrode enters on its extra row and its potential is read there
(electrode.cpp:133-150, 341-355).  Bypass resistors add to node rows
(dcfemmodelling.cpp:670-708).  Both are independent of the resistivity and
of the wavenumber, so they are built once on the host here and added on the
device after every assembly.

The reference also reads map files from its working directory
(``bypass.map``, ``electrodeBypassResistances.map``, ``contactImpedance.map``,
``contactResistance.map``); here contact impedances and bypass resistances
are arguments.  CEM electrodes made of cells, free electrodes inside cells,
reference and calibration nodes are not supported.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

MARKER_BOUND_ELECTRODE = -10000
MARKER_FIXEDVALUE_REGION = -1000000
MARKER_NODE_ELECTRODE = -99
_TOL = 1e-12


# ------------------------------------------------------------ integrals --
def _p2_mass(vertices, edges, scale, v_diag, v_off, v_adj, v_opp, e_diag, e_share, e_opp):
    """Mass matrix of a quadratic simplex from the values per node relation."""
    nv = len(vertices) + len(edges)
    m = np.empty((nv, nv))
    nvx = len(vertices)
    for i in range(nv):
        for j in range(nv):
            if i < nvx and j < nvx:
                m[i, j] = v_diag if i == j else v_off
            elif i < nvx or j < nvx:
                v, e = (i, edges[j - nvx]) if i < nvx else (j, edges[i - nvx])
                m[i, j] = v_adj if v in e else v_opp
            elif i == j:
                m[i, j] = e_diag
            else:
                shared = set(edges[i - nvx]) & set(edges[j - nvx])
                m[i, j] = e_share if shared else e_opp
    return m * scale


_TRI6_EDGES = ((0, 1), (1, 2), (2, 0))
_TET10_EDGES = ((0, 1), (0, 2), (0, 3), (1, 2), (2, 3), (1, 3))
_TRI6_U2 = _p2_mass((0, 1, 2), _TRI6_EDGES, 1.0 / 180.0, 6, -1, 0, -4, 32, 16, 16)
_TET10_U2 = _p2_mass((0, 1, 2, 3), _TET10_EDGES, 1.0 / 420.0, 6, 1, -4, -6, 32, 16, 8)


def entity_size(corners):
    """Length, area or volume from the corner positions of an entity."""
    c = np.asarray(corners, np.float64)
    if len(c) == 2:
        return float(np.linalg.norm(c[1] - c[0]))
    if len(c) == 3:
        return float(0.5 * np.linalg.norm(np.cross(c[1] - c[0], c[2] - c[0])))
    return float(abs(np.linalg.det(np.stack([c[1] - c[0], c[2] - c[0], c[3] - c[0]]))) / 6.0)


def entity_integrals(nvert, corners):
    """(u, u2) = (integral N_i, integral N_i N_j) of linear or quadratic
    Lagrange functions on an edge (2 / 3 nodes: ends, middle), a triangle
    (3 / 6 nodes) or a tetrahedron (4 / 10 nodes), in closed form; the
    reference integrates the same by exact quadrature (elementmatrix.cpp:
    48-130, 635-800).  One corner = a node: (1, 1)."""
    ncorner = len(corners)
    if ncorner == 1:
        return np.ones(1), np.ones((1, 1))
    A = entity_size(corners)
    if ncorner == 2:
        if nvert == 2:
            return A * np.array([0.5, 0.5]), (A / 6.0) * np.array([[2.0, 1.0], [1.0, 2.0]])
        return (A * np.array([1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0]),
                (A / 30.0) * np.array([[4.0, -1.0, 2.0], [-1.0, 4.0, 2.0], [2.0, 2.0, 16.0]]))
    if ncorner == 3:
        if nvert == 3:
            return np.full(3, A / 3.0), (A / 12.0) * (np.ones((3, 3)) + np.eye(3))
        return A * np.array([0.0, 0.0, 0.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0]), A * _TRI6_U2
    if nvert == 4:
        return np.full(4, A / 4.0), (A / 20.0) * (np.ones((4, 4)) + np.eye(4))
    return A * np.array([-0.05] * 4 + [0.2] * 6), A * _TET10_U2


# ------------------------------------------------------------ electrodes --
@dataclass
class ElectrodeShape:
    """One electrode or passive body: ``kind`` "node" (a node electrode or a
    bypass electrode at its first node), "cem", "passive" or "entity" (a
    point inside the cell ``entities[0]``); ``entities`` are ("b", boundary) /
    ("c", cell) pairs."""
    kind: str
    pos: np.ndarray
    node: int = -1
    entities: list = field(default_factory=list)
    size: float = 0.0
    key: int = -1


@dataclass
class ElectrodeSetup:
    """Result of the electrode search for the total-potential operator."""
    electrodes: list             # in sensor order
    passive: list                # passive bodies
    bypass_markers: list         # node markers with bypass resistors, in node order
    cem: bool                    # the matrix carries electrode rows
    n_ext: int                   # extra rows / columns
    rows: np.ndarray             # extension entries (int32), added to every assembled matrix
    cols: np.ndarray
    vals: np.ndarray
    src_row: np.ndarray          # row of each electrode's current and potential (int32)
    enode: np.ndarray            # node of each electrode, -1 for CEM electrodes (int32)
    src_center: np.ndarray       # mean electrode position (mixed boundary condition)
    search: object = None        # ert.ElectrodeSearch when an electrode lies inside a cell


def _sensor_positions(dim, sensors):
    p = np.asarray(sensors, np.float64).reshape(-1, 3).copy()
    if dim == 2:
        zvar = np.ptp(p[:, 2]) > 0 or np.max(np.abs(p[:, 2])) > 0
        yvar = np.ptp(p[:, 1]) > 0
        if zvar and not yvar and np.max(np.abs(p[:, 1])) < 1e-8:
            p[:, [1, 2]] = p[:, [2, 1]]
    return p


def has_cem_markers(mesh):
    """True when the mesh carries CEM, passive-body or bypass markers."""
    bm = np.asarray(mesh.boundary_markers)
    cm = np.asarray(mesh.cell_markers)
    nm = np.asarray(mesh.node_markers)
    return bool(np.any(bm <= MARKER_BOUND_ELECTRODE + 1)
                or np.any((cm <= MARKER_BOUND_ELECTRODE) & (cm > MARKER_FIXEDVALUE_REGION))
                or np.any(nm <= MARKER_BOUND_ELECTRODE))


def search_electrodes(mesh, sensors):
    """Electrodes in sensor order, passive bodies and bypass markers, matched
    as the reference does (CEM, then bypass, then node electrodes)."""
    dim = mesh.dim()
    nodes = np.asarray(mesh.nodes, np.float64)
    ePos = _sensor_positions(dim, sensors)
    groups: dict = {}
    bm = np.asarray(mesh.boundary_markers)
    for b in np.nonzero(bm <= MARKER_BOUND_ELECTRODE + 1)[0]:
        groups.setdefault(MARKER_BOUND_ELECTRODE - int(bm[b]), []).append(("b", int(b)))
    cm = np.asarray(mesh.cell_markers)
    for c in np.nonzero((cm <= MARKER_BOUND_ELECTRODE) & (cm > MARKER_FIXEDVALUE_REGION))[0]:
        groups.setdefault(MARKER_BOUND_ELECTRODE - int(cm[c]), []).append(("c", int(c)))
    nm = np.asarray(mesh.node_markers)
    bypass: dict = {}
    bypass_markers = []
    for i in np.nonzero(nm <= MARKER_BOUND_ELECTRODE)[0]:
        key = MARKER_BOUND_ELECTRODE - int(nm[i])
        if key in groups:
            continue
        if key not in bypass:
            bypass_markers.append(int(nm[i]))
        bypass.setdefault(key, []).append(int(i))

    def ent_nodes(kind, idx):
        return mesh.boundaries[idx] if kind == "b" else mesh.cells[idx]

    def ent_corners(kind, idx):
        nc = dim if kind == "b" else dim + 1
        return nodes[ent_nodes(kind, idx)[:nc]]

    cem, passive = [], []
    for key in sorted(groups):
        ents = groups[key]
        size = sum(entity_size(ent_corners(k, i)) for k, i in ents)
        uniq = sorted({int(v) for k, i in ents for v in ent_nodes(k, i)})
        shape = ElectrodeShape("cem" if key >= 0 else "passive", nodes[uniq].sum(axis=0) / len(uniq),
                               entities=ents, size=size, key=key)
        (cem if key >= 0 else passive).append(shape)
    byp = [(key, bypass[key]) for key in sorted(bypass)]
    node_el = list(np.nonzero(nm == MARKER_NODE_ELECTRODE)[0])
    electrodes = []
    for i, p in enumerate(ePos):
        hit = None
        for j, el in enumerate(cem):
            if np.linalg.norm(p - el.pos) < math.sqrt(el.size) * 2.0 or el.key == i:
                hit = cem.pop(j)
                hit.pos = p.copy()
                break
        if hit is None:
            for j, (key, nlist) in enumerate(byp):
                if np.linalg.norm(p - nodes[nlist[0]]) < 0.01:
                    byp.pop(j)
                    hit = ElectrodeShape("node", nodes[nlist[0]].copy(), node=nlist[0])
                    break
        if hit is None:
            for j, nd in enumerate(node_el):
                if np.linalg.norm(p - nodes[nd]) < 0.01:
                    node_el.pop(j)
                    hit = ElectrodeShape("node", nodes[nd].copy(), node=int(nd))
                    break
        if hit is None:
            # no electrode node: the cell that holds the sensor (ElectrodeShapeEntity,
            # dcfemmodelling.cpp:924-937)
            from .ert import find_cell
            cell = find_cell(mesh, p)
            if cell < 0:
                raise ValueError(f"There is a requested electrode that does not match the given mesh: sensor {i} "
                                 f"at {p}")
            hit = ElectrodeShape("entity", p.copy(), entities=[("c", int(cell))])
        electrodes.append(hit)
    return electrodes, passive, bypass_markers, ent_nodes, ent_corners


def electrode_setup(mesh, sensors, contact_impedance=None, bypass_resistance=None):
    """Electrodes and the matrix extension of the total-potential operator.

    contact_impedance: one value per electrode, then per passive body (Ohm m^2,
    default 1; setContactImpedances); point electrodes always use 1.
    bypass_resistance: {node marker: Ohm} (default 1e-6 Ohm)."""
    electrodes, passive, bypass_markers, ent_nodes, ent_corners = search_electrodes(mesh, sensors)
    entity = [e for e in electrodes if e.kind == "entity"]
    if entity and (any(e.kind == "cem" for e in electrodes) or passive):
        raise NotImplementedError("electrodes inside cells together with complete-electrode-model electrodes")
    if any(k == "c" for el in electrodes + passive if el.kind != "entity" for k, _ in el.entities):
        raise NotImplementedError("CEM electrodes made of cells (cell marker -10000 - i) are not supported; "
                                  "mark the electrode's boundaries instead")
    nn = mesh.nodeCount()
    nE = len(electrodes)
    cem = any(e.kind == "cem" for e in electrodes) or len(passive) > 0
    rows, cols, vals = [], [], []
    n_ext = 0
    if cem:
        elecs = electrodes + passive
        n_ext = len(elecs)
        z_all = np.ones(n_ext)
        if contact_impedance is not None:
            z = np.asarray(contact_impedance, np.float64).ravel()
            if len(z) != n_ext:
                raise ValueError(f"contact impedances: {len(z)} values for {n_ext} electrodes and passive bodies")
            z_all = z
        for j, el in enumerate(elecs):
            mat = nn + j
            z = float(z_all[j])
            area = el.size
            if area < _TOL:          # a point electrode: unit contact
                z, area = 1.0, 1.0
            ents = [("n", el.node)] if el.kind == "node" else el.entities
            for kind, idx in ents:
                if kind == "n":
                    ids = np.array([idx])
                    u, u2 = entity_integrals(1, np.zeros((1, 3)))
                else:
                    ids = np.asarray(ent_nodes(kind, idx))
                    u, u2 = entity_integrals(len(ids), ent_corners(kind, idx))
                for i, nd in enumerate(ids):
                    rows += [int(nd), mat]
                    cols += [mat, int(nd)]
                    vals += [-u[i] / z, -u[i] / z]
                for i, a in enumerate(ids):
                    for k, b in enumerate(ids):
                        rows.append(int(a))
                        cols.append(int(b))
                        vals.append(u2[i, k] / z)
            rows.append(mat)
            cols.append(mat)
            vals.append(area / z)
    res = bypass_resistance or {}
    nm = np.asarray(mesh.node_markers)
    for mk in bypass_markers:
        nl = np.nonzero(nm == mk)[0]
        g = 1.0 / float(res.get(mk, 1e-6))
        for a1, a2 in zip(nl[:-1], nl[1:]):
            rows += [int(a1), int(a2), int(a1), int(a2)]
            cols += [int(a1), int(a2), int(a2), int(a1)]
            vals += [g, g, -g, -g]
    if cem:
        src_row = nn + np.arange(nE)
    else:
        src_row = np.array([e.node for e in electrodes])
    enode = np.array([e.node if e.kind == "node" else -1 for e in electrodes])
    center = sum(e.pos for e in electrodes) / nE
    search = None
    if entity:
        from .ert import ElectrodeSearch
        search = ElectrodeSearch(enode.astype(np.int32),
                                 np.array([e.entities[0][1] if e.kind == "entity" else -1 for e in electrodes],
                                          np.int32),
                                 np.array([e.pos for e in electrodes], np.float64))
    return ElectrodeSetup(electrodes, passive, bypass_markers, cem, n_ext, np.asarray(rows, np.int32),
                          np.asarray(cols, np.int32), np.asarray(vals, np.float64), src_row.astype(np.int32),
                          enode.astype(np.int32), np.asarray(center, np.float64), search)


def mark_cem_electrodes(mesh, positions, radius, passive=None):
    """Copy of ``mesh`` whose surface boundaries (marker -1) within ``radius``
    (horizontal distance of every boundary node) of ``positions[i]`` carry
    the CEM marker -10000 - i; ``passive``: a list of (position, radius) for
    passive bodies (-9999).  Node markers of the electrodes are reset to 0."""
    from .mesh import Mesh
    bm = np.array(mesh.boundary_markers, np.int32)
    nm = np.array(mesh.node_markers, np.int32)
    dim = mesh.dim()
    hor = [0] if dim == 2 else [0, 1]
    nodes = np.asarray(mesh.nodes)
    surf = np.nonzero(bm == -1)[0]

    def within(center, r):
        c = np.asarray(center, np.float64).ravel()
        d = np.linalg.norm(nodes[mesh.boundaries[surf]][:, :, hor] - c[hor][None, None, :], axis=2)
        return surf[np.all(d <= r + 1e-12, axis=1)]

    for i, p in enumerate(np.asarray(positions, np.float64).reshape(len(positions), -1)):
        pp = np.zeros(3)
        pp[:len(p)] = p
        sel = within(pp, radius)
        if len(sel) == 0:
            raise ValueError(f"no surface boundary within {radius} of electrode {i}")
        bm[sel] = MARKER_BOUND_ELECTRODE - i
    for p, r in (passive or []):
        pp = np.zeros(3)
        pp[:len(p)] = p
        sel = within(pp, r)
        sel = sel[bm[sel] == -1]
        bm[sel] = MARKER_BOUND_ELECTRODE + 1
    nm[nm == MARKER_NODE_ELECTRODE] = 0
    return Mesh(dim, nodes.copy(), mesh.cells.copy(), mesh.cell_markers.copy(), nm, mesh.boundaries.copy(), bm,
                mesh.boundary_cells.copy(), check=False)
