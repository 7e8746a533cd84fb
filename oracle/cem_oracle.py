"""Test infrastructure only -- the oracle for the total-potential operator.

An FP64 CPU restatement (numpy/scipy) of the reference's
DCMultiElectrodeModelling (pyGIMLi ERTModelling(sr=False)): total
potentials for unit point currents, no singularity removal, plus the two
constant extensions of its system matrix that only this operator builds --
the complete electrode model (CEM) and bypass resistors.  It is the checker
for the CUDA product path; the product never imports it.  It is pinned to
the reference's own compiled C++ (oracle/_ref) by tests/test_cem.py and the
fixtures tests/golden/ert*_tp_*.npz, tests/golden/ert*_cem_*.npz.

Reference code restated (paths inside pyGIMLi):

  electrode search   core/src/bert/dcfemmodelling.cpp:790-1030 (CEM faces
                     and cells 804-820, bypass nodes 823-836, matching order
                     CEM -> bypass -> node electrodes 863-947, passive
                     bodies 978-985)
  electrode shapes   core/src/bert/electrode.cpp:81-100 (node), 191-193
                     (nodes with bypass), 287-318 (domain: size, position),
                     341-355 (domain right-hand side)
  CEM extension      core/src/bert/dcfemmodelling.cpp:315-414
                     assembleCompleteElectrodeModel_, 1786-1831 (calculateK_)
  entity integrals   core/src/elementmatrix.cpp:48-130 (u, u2 by quadrature),
                     635-800 (rules per entity type)
  bypass resistors   core/src/bert/dcfemmodelling.cpp:601-709
  total potentials   core/src/bert/dcfemmodelling.cpp:1756-1929 calculateK_
  k-sum / collect    core/src/bert/dcfemmodelling.cpp:1669-1730, 1632-1649;
                     with CEM the electrode potentials are those of the last
                     wavenumber only (potentialsCEM_ is overwritten per
                     wavenumber, 1829 and 1912, and collected unweighted)
  response           core/src/bert/dcfemmodelling.cpp:1085-1197
  Jacobian           core/src/bert/bertJacobian.cpp:267-421 on the node
                     rows of the sub-potentials (1906-1908)

Not restated: the map files the reference reads from the working directory
(bypass.map, electrodeBypassResistances.map, contactImpedance.map,
contactResistance.map) -- their values enter here as arguments; a
reference electrode together with CEM electrodes.

Reference and calibration nodes, Neumann domains and homogeneous Dirichlet
boundaries follow ert_oracle.BoundarySetup: Dirichlet rows cleaned before
the extensions (dcfemBoundaryAssembleStiffnessMatrix,
core/src/bert/dcfemmodelling.cpp:279-298), calibration rows after them
(1835), the pattern of electrode e carrying +1 there and -1 at the reference
electrode (1515-1523, 1862-1864).
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from ert_oracle import (TOLERANCE, BoundarySetup, Problem, _p2_shape, _rule_tet_deg4, _rule_tri_deg4, boundary_center_normal,
                        boundary_mass, element_matrices, find_cell, mixed_bc_alpha, sparsity_pattern)

MARKER_BOUND_ELECTRODE = -10000
MARKER_FIXEDVALUE_REGION = -1000000
MARKER_NODE_ELECTRODE = -99


# ------------------------------------------------------ entity integrals --
def _edge_rule():
    """3-point Gauss-Legendre on [0, 1] (exact to degree 5)."""
    x, w = np.polynomial.legendre.leggauss(3)
    return 0.5 * (x + 1.0), 0.5 * w


def _entity_shape(dim_e, nvert, pts):
    """Shape functions of an entity at reference points (Q x nvert):
    dim_e 1 = edge (2 or 3 nodes: ends, middle), 2 = triangle (3 or 6),
    3 = tetrahedron (4 or 10), in the mesh's node order."""
    if dim_e == 1:
        t = pts
        if nvert == 2:
            return np.column_stack([1.0 - t, t])
        return np.column_stack([(1.0 - t) * (1.0 - 2.0 * t), t * (2.0 * t - 1.0), 4.0 * t * (1.0 - t)])
    if nvert == dim_e + 1:
        return np.asarray(pts)
    return _p2_shape(dim_e, np.asarray(pts))


def entity_size(xyz):
    """Length / area / volume of an entity from its corner nodes."""
    m = len(xyz)
    if m == 1:
        return 1.0
    if m == 2:
        return float(np.linalg.norm(xyz[1] - xyz[0]))
    if m == 3:
        return float(0.5 * np.linalg.norm(np.cross(xyz[1] - xyz[0], xyz[2] - xyz[0])))
    return float(abs(np.linalg.det(np.stack([xyz[1] - xyz[0], xyz[2] - xyz[0], xyz[3] - xyz[0]]))) / 6.0)


def entity_integrals(dim_e, xyz_corner, nvert):
    """(u, u2): integrals of N_i and N_i N_j over one entity (a node, an
    edge, a triangle or a tetrahedron), by quadrature exact for the degree."""
    if dim_e == 0:
        return np.ones(1), np.ones((1, 1))
    if dim_e == 1:
        pts, w = _edge_rule()
    elif dim_e == 2:
        pts, w = _rule_tri_deg4()
    else:
        pts, w = _rule_tet_deg4()
    N = _entity_shape(dim_e, nvert, pts)
    A = entity_size(xyz_corner)
    return A * (w @ N), A * np.einsum("q,qi,qj->ij", w, N, N)


# ------------------------------------------------------- electrode search --
class Electrode:
    """kind: 'node' (node electrode or bypass electrode at its first node),
    'cem' (electrode faces or cells), 'passive' (passive CEM body)."""

    def __init__(self, kind, pos, node=-1, entities=(), size=0.0, key=-1):
        self.kind, self.pos, self.node = kind, np.asarray(pos, float), node
        self.entities, self.size, self.key = list(entities), size, key


def _entity_dim(mesh, kind, idx):
    if kind == "b":
        return mesh.dim() - 1
    return mesh.dim()


def _entity_nodes(mesh, kind, idx):
    return mesh.boundaries[idx] if kind == "b" else mesh.cells[idx]


def search_electrodes(mesh, sensors):
    """Electrodes in data order, passive bodies, bypass markers in node order
    (dcfemmodelling.cpp:790-1030)."""
    dim = mesh.dim()
    ePos = np.asarray(sensors, np.float64).reshape(-1, 3).copy()
    if dim == 2:
        zvar = np.ptp(ePos[:, 2]) > 0 or np.max(np.abs(ePos[:, 2])) > 0
        yvar = np.ptp(ePos[:, 1]) > 0
        if zvar and not yvar and np.max(np.abs(ePos[:, 1])) < 1e-8:
            ePos[:, [1, 2]] = ePos[:, [2, 1]]
    faces = {}
    for b, mk in enumerate(mesh.boundary_markers):
        if mk <= MARKER_BOUND_ELECTRODE + 1:
            faces.setdefault(MARKER_BOUND_ELECTRODE - int(mk), []).append(("b", b))
    for c, mk in enumerate(mesh.cell_markers):
        if MARKER_FIXEDVALUE_REGION < mk <= MARKER_BOUND_ELECTRODE:
            faces.setdefault(MARKER_BOUND_ELECTRODE - int(mk), []).append(("c", c))
    bypass, bypass_markers = {}, []
    for i, mk in enumerate(mesh.node_markers):
        key = MARKER_BOUND_ELECTRODE - int(mk)
        if mk <= MARKER_BOUND_ELECTRODE and key not in faces:
            if key not in bypass:
                bypass_markers.append(int(mk))
            bypass.setdefault(key, []).append(i)
    cem, passive = [], []
    for key in sorted(faces):
        ents = faces[key]
        size = sum(entity_size(mesh.nodes[_entity_nodes(mesh, k, i)][:_entity_dim(mesh, k, i) + 1])
                   for k, i in ents)
        nodes = sorted({int(v) for k, i in ents for v in _entity_nodes(mesh, k, i)})
        pos = mesh.nodes[nodes].sum(axis=0) / len(nodes)
        el = Electrode("cem" if key >= 0 else "passive", pos, entities=ents, size=size, key=key)
        (cem if key >= 0 else passive).append(el)
    byp = [(key, bypass[key]) for key in sorted(bypass)]
    src = list(np.nonzero(mesh.node_markers == MARKER_NODE_ELECTRODE)[0])
    electrodes = []
    for i, p in enumerate(ePos):
        hit = None
        for j, el in enumerate(cem):
            if np.linalg.norm(p - el.pos) < math.sqrt(el.size) * 2.0 or el.key == i:
                hit = cem.pop(j)
                hit.pos = p.copy()
                break
        if hit is None:
            for j, (key, nodes) in enumerate(byp):
                if np.linalg.norm(p - mesh.nodes[nodes[0]]) < 0.01:
                    byp.pop(j)
                    hit = Electrode("node", mesh.nodes[nodes[0]], node=nodes[0])
                    break
        if hit is None:
            for j, nd in enumerate(src):
                if np.linalg.norm(p - mesh.nodes[nd]) < 0.01:
                    src.pop(j)
                    hit = Electrode("node", mesh.nodes[nd], node=int(nd))
                    break
        if hit is None:
            # no electrode node: the cell that holds the sensor (ElectrodeShapeEntity)
            cell, wts = find_cell(mesh, p)
            if cell < 0:
                raise ValueError("There is a requested electrode that does not match the given mesh.")
            hit = Electrode("entity", p.copy())
            hit.rows, hit.wts = mesh.cells[cell].astype(np.int64), wts
        electrodes.append(hit)
    return electrodes, passive, bypass_markers


# ---------------------------------------------------- matrix extensions --
def cem_entries(mesh, electrodes, passive, contact_impedance=None):
    """Entries of the complete electrode model (assembleCompleteElectrodeModel_,
    dcfemmodelling.cpp:315-414) as {(row, col): value} plus the assigned
    diagonal of the electrode rows; rows nNodes + j for elecs[j] (electrodes,
    then passive bodies)."""
    nn = len(mesh.nodes)
    elecs = list(electrodes) + list(passive)
    z_all = np.ones(len(elecs)) if contact_impedance is None else np.asarray(contact_impedance, float)
    add, diag = {}, {}

    def acc(r, c, v):
        add[(r, c)] = add.get((r, c), 0.0) + v

    for j, el in enumerate(elecs):
        mat = nn + j
        sum_area = el.size
        z = float(z_all[j])
        if el.kind == "node":
            ents = [("n", el.node)]
        else:
            ents = el.entities
        if sum_area < TOLERANCE:
            z, sum_area = 1.0, 1.0
        for kind, idx in ents:
            if kind == "n":
                ids = np.array([idx])
                u, u2 = entity_integrals(0, None, 1)
            else:
                ids = _entity_nodes(mesh, kind, idx)
                de = _entity_dim(mesh, kind, idx)
                u, u2 = entity_integrals(de, mesh.nodes[ids[:de + 1]], len(ids))
            for i, nd in enumerate(ids):
                acc(int(nd), mat, -u[i] / z)
                acc(mat, int(nd), -u[i] / z)
            for i, a in enumerate(ids):
                for k, b in enumerate(ids):
                    acc(int(a), int(b), u2[i, k] / z)
        diag[mat] = 1.0 if abs(sum_area) < TOLERANCE else sum_area / z
    return add, diag, len(elecs)


def bypass_entries(mesh, bypass_markers, resistance=None):
    """Bypass resistors between consecutive nodes of each bypass marker
    (dcfemmodelling.cpp:670-708): 1 / R on both diagonals, -1 / R off."""
    add = {}
    resistance = resistance or {}
    for mk in bypass_markers:
        nodes = np.nonzero(mesh.node_markers == mk)[0]
        R = float(resistance.get(mk, 1e-6))
        for a1, a2 in zip(nodes[:-1], nodes[1:]):
            v = 1.0 / R
            for (r, c), s in (((a1, a1), v), ((a2, a2), v), ((a1, a2), -v), ((a2, a1), -v)):
                add[(int(r), int(c))] = add.get((int(r), int(c)), 0.0) + s
    return add


# ------------------------------------------------------------ operator --
class TotalPotentialProblem:
    """Mesh + electrodes + scheme of the total-potential operator."""

    def __init__(self, mesh, sensors, abmn, kfac, k, w, contact_impedance=None, bypass_resistance=None,
                 dipole=False):
        self.mesh = mesh
        self.dipole = bool(dipole)  # patterns of the dipole current pattern (ert_oracle.BoundarySetup)
        self.dim = mesh.dim()
        nodes = mesh.nodes
        self.n = len(nodes)
        self.abmn = np.asarray(abmn, np.int64).reshape(-1, 4)
        self.kfac = np.asarray(kfac, np.float64)
        self.k = np.asarray(k, np.float64)
        self.w = np.asarray(w, np.float64)
        self.rowptr, self.cols = sparsity_pattern(self.n, mesh.cells)
        self.K, self.M = element_matrices(self.dim, nodes, mesh.cells)
        self.electrodes, self.passive, self.bypass_markers = search_electrodes(mesh, sensors)
        self.nE = len(self.electrodes)
        self.src_center = sum(e.pos for e in self.electrodes) / self.nE
        self.cem = any(e.kind == "cem" for e in self.electrodes) or len(self.passive) > 0
        ext = {}
        diag = {}
        self.n_ext = 0
        if self.cem:
            ext, diag, self.n_ext = cem_entries(mesh, self.electrodes, self.passive, contact_impedance)
        for key, v in bypass_entries(mesh, self.bypass_markers, bypass_resistance).items():
            ext[key] = ext.get(key, 0.0) + v
        self.N = self.n + self.n_ext
        self.ext = ext
        self.ext_diag = diag
        if self.cem:
            self.src_row = self.n + np.arange(self.nE)
        else:
            self.src_row = np.array([e.node for e in self.electrodes], np.int64)
        # source / collect weights per electrode: its row, or an entity electrode's cell nodes
        self.erows = [getattr(e, "rows", None) if e.kind == "entity" else np.array([self.src_row[i]])
                      for i, e in enumerate(self.electrodes)]
        self.ewts = [getattr(e, "wts", None) if e.kind == "entity" else np.ones(1)
                     for e in self.electrodes]
        bm = mesh.boundary_markers
        self.mixed = np.nonzero(bm == -2)[0]
        bnd = mesh.boundaries[self.mixed]
        self.bnd_cell = mesh.boundary_cells[self.mixed]
        self.bnd_mass = boundary_mass(self.dim, nodes, bnd)
        bc, bn = boundary_center_normal(self.dim, nodes, bnd)
        self.alpha = [mixed_bc_alpha(self.dim, bc, bn, self.src_center, kk) for kk in self.k]
        self.bnd_nodes = bnd
        Problem._slot_maps(self)
        self.epos = np.array([e.pos for e in self.electrodes], np.float64)
        Problem._patterns(self)
        self.dirichlet = self.bc.dirichlet
        if self.sink is not None and self.n_ext:
            raise NotImplementedError("a reference electrode with complete-electrode-model electrodes")

    def matrix(self, rho_cell, kidx):
        """FEM matrix (domain, mixed boundaries) plus the extensions, N x N."""
        kk = self.k[kidx]
        vals = np.zeros(len(self.cols))
        Se = self.M * (kk * kk) + self.K if kk > 0.0 else self.K
        valid = np.abs(rho_cell) > TOLERANCE
        contrib = Se * (1.0 / np.where(valid, rho_cell, 1.0))[:, None, None]
        contrib[~valid] = 0.0
        np.add.at(vals, self.cell_slot.ravel(), contrib.ravel())
        if len(self.mixed):
            bc = self.bnd_mass * (self.alpha[kidx] / rho_cell[self.bnd_cell])[:, None, None]
            np.add.at(vals, self.bnd_slot.ravel(), bc.ravel())
        diag_slot = Problem._diag_slots(self)
        if len(self.dirichlet):
            Problem._clean_rows_cols(self, vals, self.dirichlet, diag_slot)
        A = sp.csr_matrix((vals, self.cols, self.rowptr), shape=(self.n, self.n))
        A = sp.block_diag([A, sp.csr_matrix((self.n_ext, self.n_ext))]).tolil() if self.n_ext else A.tolil()
        for (r, c), v in self.ext.items():
            A[r, c] += v
        for r, v in self.ext_diag.items():
            A[r, r] = v
        for r in self.calib:
            A[r, :] = 0.0
            A[:, r] = 0.0
            A[r, r] = 1.0
        return A.tocsr()

    def solve(self, rho_cell):
        """u[kIdx, e, row] for a unit current at each electrode's source row."""
        nK = len(self.k)
        u = np.zeros((nK, self.nE, self.N))
        for ki in range(nK):
            lu = spla.splu(self.matrix(rho_cell, ki).tocsc(), permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0)
            for e in range(self.nE):
                rhs = np.zeros(self.N)
                rhs[self.erows[e]] += self.ewts[e]
                if self.sink is not None:
                    rhs[self.sink[0]] -= self.sink[1]
                u[ki, e] = lu.solve(rhs)
        return u

    def collect(self, u):
        if self.cem:
            return u[-1][:, self.src_row].copy()
        sol = np.einsum("k,ken->en", self.w, u)
        return np.stack([sol[:, r] @ w for r, w in zip(self.erows, self.ewts)], axis=1)

    def calculate(self, rho_cell):
        """Signed voltages of the data for a unit current (Problem.calculate)."""
        return Problem.calculate(self, rho_cell)

    def response(self, rho_cell):
        if np.min(rho_cell) < TOLERANCE:
            raise ValueError("response for model with negative or zero resistivity is not defined")
        u = self.solve(rho_cell)
        U = self.collect(u)
        r = np.rint(Problem.data_u(self, U) / 1e-10) * 1e-10
        rr = np.rint(Problem.data_u(self, U, True) / 1e-10) * 1e-10
        return np.sqrt(np.abs(r * self.kfac * (rr * self.kfac))), u

    def jacobian(self, u, model, n_params=None):
        return Problem.jacobian(self, u[:, :, :self.n], model, n_params)
