"""Test infrastructure only -- the oracle.

An FP64 CPU restatement (numpy/scipy) of the reference's ERT forward
operator with singularity removal and its reciprocity Jacobian.  It is the
checker for the CUDA product path and the CPU baseline timed beside it; the
product never imports it.  It is pinned against the reference's own compiled
C++ (oracle/_ref, via oracle/ref_driver.py) by tests/test_oracle.py and the
fixtures in tests/golden/.

Each step cites the reference code it restates (paths inside pyGIMLi):

  pattern            core/src/sparsematrix.h:966-1024 buildSparsityPattern
  element matrices   core/src/elementmatrix.cpp:683-796 (u2), 798-870 and
                     1036-1041 (ux2uy2uz2: triangle closed form, tetrahedron
                     one-point rule), core/src/integration.cpp (rules)
  domain assembly    core/src/bert/dcfemmodelling.cpp:163-228
  mixed boundary     core/src/bert/dcfemmodelling.cpp:243-299 and 430-506
  Bessel K0/K1       core/src/numericbase.h:79-175 (Abramowitz & Stegun
                     9.8.1-9.8.8 polynomial approximations)
  primary potential  core/src/bert/bertMisc.cpp:186-271 exactDCSolution,
                     core/src/bert/electrode.cpp:154-197 setSingValue
  source resistivity core/src/bert/electrode.cpp:102-127 geomMeanCellAttributes
  SR solve           core/src/bert/dcfemmodelling.cpp:2152-2296 calculateK
  k-sum              core/src/bert/dcfemmodelling.cpp:1697-1729
  collect / data     core/src/bert/datamap.cpp:57-98, 159-231
  response           core/src/bert/dcfemmodelling.cpp:1133-1196
  Jacobian           core/src/bert/bertJacobian.cpp:70-119 (calc2),
                     267-421; scaling dcfemmodelling.cpp:1377-1384
  electrode search   core/src/bert/dcfemmodelling.cpp:790-1030
  Neumann domains    core/src/bert/dcfemmodelling.cpp:711-773 (detection),
                     1011-1073 (reference electrode, calibration nodes),
                     1515-1523 (current patterns), 2182-2192 and 2281-2283
                     (calibration rows), 2236-2266 (source resistivity of a
                     pattern); homogeneous Dirichlet boundaries 279-298 and
                     142-154; reference-electrode data datamap.cpp:203-214
  model mapping      core/src/modellingbase.cpp:401-497,
                     core/src/mesh.cpp:2247-2316 prolongateEmptyCellsValues
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

TOLERANCE = 1e-12
PI = math.pi
MARKER_BOUND_HOMOGEN_NEUMANN = -1
MARKER_BOUND_MIXED = -2
MARKER_BOUND_HOMOGEN_DIRICHLET = -3
MARKER_BOUND_DIRICHLET = -4
MARKER_NODE_REFERENCEELECTRODE = -999
MARKER_NODE_CALIBRATION = -1000


class BoundarySetup:
    """Boundary conditions and current patterns of a mesh
    (updateMeshDependency_, core/src/bert/dcfemmodelling.cpp:711-773;
    searchElectrodes_, 799-802 and 1011-1073):

    neumann    no mixed and no Dirichlet boundary (in 2-D only the topography
               flag follows from it)
    topography a Neumann-boundary centre off the first one's height, or a
               Neumann domain (any dimension)
    dirichlet  nodes of homogeneous Dirichlet boundaries (-3), sorted
    calib      calibration nodes of a 3-D Neumann domain: node marker -1000,
               else node 0
    ref_node   the first node with marker -999 (-1: none); its patterns
               (e, ref) hold for every domain
    ref_elec   a 3-D Neumann domain without reference node: the last
               electrode (its own pattern is empty), else -1

    dipole=True (the dipole current pattern, setDipoleCurrentPattern): no
    reference at all, since createCurrentPattern (1488-1513) pairs the data's
    own a and b electrodes and searchElectrodes_ picks no last-electrode
    reference then (1054); a pole datum (b = -1) of a closed domain drains
    its current at the calibration nodes.
    """

    def __init__(self, mesh, n_elec, dipole=False):
        bm = np.asarray(mesh.boundary_markers)
        if np.any(bm == MARKER_BOUND_DIRICHLET):
            raise NotImplementedError("inhomogeneous Dirichlet boundaries (-4) are not implemented")
        self.neumann = not np.any((bm == MARKER_BOUND_MIXED) | (bm == MARKER_BOUND_HOMOGEN_DIRICHLET))
        neu = np.nonzero(bm == MARKER_BOUND_HOMOGEN_NEUMANN)[0]
        topo = False
        if len(neu):
            cz = mesh.nodes[mesh.boundaries[neu]].mean(axis=1)[:, mesh.dim() - 1]
            topo = bool(np.any(cz != cz[0]))
        self.topography = topo or self.neumann
        dnodes = mesh.boundaries[bm == MARKER_BOUND_HOMOGEN_DIRICHLET]
        self.dirichlet = np.unique(dnodes.ravel()).astype(np.int64) if len(dnodes) else np.zeros(0, np.int64)
        nm = np.asarray(mesh.node_markers)
        refs = np.nonzero(nm == MARKER_NODE_REFERENCEELECTRODE)[0]
        self.ref_node = int(refs[0]) if len(refs) else -1
        self.ref_elec = -1
        neumann3 = self.neumann and mesh.dim() == 3
        if neumann3:
            cal = np.nonzero(nm == MARKER_NODE_CALIBRATION)[0]
            self.calib = cal.astype(np.int64) if len(cal) else np.zeros(1, np.int64)
            if self.ref_node < 0 and n_elec > 0 and not dipole:
                self.ref_elec = n_elec - 1
        else:
            self.calib = np.zeros(0, np.int64)
        if dipole:
            self.ref_node = -1
        self.clean = np.union1d(self.dirichlet, self.calib).astype(np.int64)


def node_min_radius(mesh, nd):
    """Smallest distance from node nd to the nodes of its cells."""
    cs = np.nonzero(np.any(mesh.cells == nd, axis=1))[0]
    nb = np.setdiff1d(np.unique(mesh.cells[cs]), [nd])
    return float(np.min(np.linalg.norm(mesh.nodes[nb] - mesh.nodes[nd], axis=1))), cs


# ---------------------------------------------------------------- Bessel --
def besselI0(x):
    x = np.asarray(x, dtype=np.float64)
    ax = np.abs(x)
    out = np.empty_like(ax)
    s = ax < 3.75
    y = x[s] / 3.75
    y = y * y
    out[s] = 1.0 + y * (3.5156229 + y * (3.0899424 + y * (1.2067492 + y * (0.2659732 + y * (
        0.360768e-1 + y * 0.45813e-2)))))
    a = ax[~s]
    y = 3.75 / a
    out[~s] = (np.exp(a) / np.sqrt(a)) * (0.39894228 + y * (0.1328592e-1 + y * (0.225319e-2 + y * (
        -0.157565e-2 + y * (0.916281e-2 + y * (-0.2057706e-1 + y * (0.2635537e-1 + y * (
            -0.1647633e-1 + y * 0.392377e-2))))))))
    return out


def besselI1(x):
    x = np.asarray(x, dtype=np.float64)
    ax = np.abs(x)
    out = np.empty_like(ax)
    s = ax < 3.75
    y = x[s] / 3.75
    y = y * y
    out[s] = ax[s] * (0.5 + y * (0.87890594 + y * (0.51498869 + y * (0.15084934 + y * (
        0.2658733e-1 + y * (0.301532e-2 + y * 0.32411e-3))))))
    a = ax[~s]
    y = 3.75 / a
    r = 0.2282967e-1 + y * (-0.2895312e-1 + y * (0.1787654e-1 - y * 0.420059e-2))
    r = 0.39894228 + y * (-0.3988024e-1 + y * (-0.362018e-2 + y * (0.163801e-2 + y * (
        -0.1031555e-1 + y * r))))
    out[~s] = r * (np.exp(a) / np.sqrt(a))
    return np.where(x < 0.0, -out, out)


def besselK0(x):
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    out = np.empty_like(x)
    s = x <= 2.0
    xs = x[s]
    y = xs * xs / 4.0
    out[s] = (-np.log(xs / 2.0) * besselI0(xs)) + (-0.57721566 + y * (0.42278420 + y * (
        0.23069756 + y * (0.3488590e-1 + y * (0.262698e-2 + y * (0.10750e-3 + y * 0.74e-5))))))
    xl = x[~s]
    y = 2.0 / xl
    out[~s] = (np.exp(-xl) / np.sqrt(xl)) * (1.25331414 + y * (-0.7832358e-1 + y * (
        0.2189568e-1 + y * (-0.1062446e-1 + y * (0.587872e-2 + y * (-0.251540e-2 + y * 0.53208e-3))))))
    return out


def besselK1(x):
    x = np.atleast_1d(np.asarray(x, dtype=np.float64))
    out = np.empty_like(x)
    s = x <= 2.0
    xs = x[s]
    y = xs * xs / 4.0
    out[s] = (np.log(xs / 2.0) * besselI1(xs)) + (1.0 / xs) * (1.0 + y * (0.15443144 + y * (
        -0.67278579 + y * (-0.18156897 + y * (-0.1919402e-1 + y * (-0.110404e-2 + y * (-0.4686e-4)))))))
    xl = x[~s]
    y = 2.0 / xl
    out[~s] = (np.exp(-xl) / np.sqrt(xl)) * (1.25331414 + y * (0.23498619 + y * (-0.3655620e-1 + y * (
        0.1504268e-1 + y * (-0.780353e-2 + y * (0.325614e-2 + y * (-0.68245e-3)))))))
    return out


# ------------------------------------------------------------- geometry --
_TET10_EDGES = ((0, 1), (0, 2), (0, 3), (1, 2), (2, 3), (3, 1))
_TRI6_EDGES = ((0, 1), (1, 2), (2, 0))


def _p2_shape(dim, lam):
    """P2 Lagrange functions at barycentric points lam (Q x dim+1): vertex
    l(2l-1), edge 4 l_a l_b in Tetrahedron10 / Triangle6 order."""
    edges = _TET10_EDGES if dim == 3 else _TRI6_EDGES
    vert = lam * (2.0 * lam - 1.0)
    edge = np.stack([4.0 * lam[:, a] * lam[:, b] for a, b in edges], axis=1)
    return np.concatenate([vert, edge], axis=1)


def _p2_grad(dim, lam, g):
    """Gradients (C x Q x nv x 3) of the P2 functions; g: barycentric gradients C x (dim+1) x 3."""
    edges = _TET10_EDGES if dim == 3 else _TRI6_EDGES
    out = [(4.0 * lam[None, :, i, None] - 1.0) * g[:, None, i, :] for i in range(dim + 1)]
    for a, b in edges:
        out.append(4.0 * (lam[None, :, b, None] * g[:, None, a, :] + lam[None, :, a, None] * g[:, None, b, :]))
    return np.stack(out, axis=2)


def _rule_tri_deg4():
    """6-point degree-4 triangle rule (Dunavant)."""
    a1, b1, w1 = 0.816847572980458513080, 0.091576213509770743460, 0.109951743655321868504
    a2, b2, w2 = 0.108103018168070227360, 0.445948490915964886320, 0.223381589678011464830
    pts, w = [], []
    for a, b, ww in ((a1, b1, w1), (a2, b2, w2)):
        for q in range(3):
            lam = [b, b, b]
            lam[q] = a
            pts.append(lam)
            w.append(ww)
    return np.array(pts), np.array(w)


def _rule_tet_deg4():
    """Keast's 11-point degree-4 tetrahedron rule (weights sum to 1)."""
    sq = math.sqrt(5.0 / 14.0)
    ca, cb = (1.0 + sq) / 4.0, (1.0 - sq) / 4.0
    pts = [[0.25] * 4]
    w = [-74.0 / 5625.0 * 6.0]
    for q in range(4):
        lam = [1.0 / 14.0] * 4
        lam[q] = 11.0 / 14.0
        pts.append(lam)
        w.append(343.0 / 45000.0 * 6.0)
    for a, b in ((0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)):
        lam = [cb] * 4
        lam[a] = lam[b] = ca
        pts.append(lam)
        w.append(56.0 / 2250.0 * 6.0)
    return np.array(pts), np.array(w)


def _bary_gradients(dim, p):
    if dim == 2:
        x1, x2, x3 = p[:, 0, 0], p[:, 1, 0], p[:, 2, 0]
        y1, y2, y3 = p[:, 0, 1], p[:, 1, 1], p[:, 2, 1]
        det = (x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1)
        g = np.zeros((len(p), 3, 3))
        g[:, 1, 0] = (y3 - y1) / det
        g[:, 1, 1] = -(x3 - x1) / det
        g[:, 2, 0] = -(y2 - y1) / det
        g[:, 2, 1] = (x2 - x1) / det
        g[:, 0] = -(g[:, 1] + g[:, 2])
        return g, np.abs(det) / 2.0
    Jm = np.stack([p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]], axis=2)
    inv = np.linalg.inv(Jm)
    g = np.empty((len(p), 4, 3))
    g[:, 1:, :] = inv
    g[:, 0, :] = -inv.sum(axis=1)
    return g, np.abs(np.linalg.det(Jm)) / 6.0


def element_matrices_p2(dim, nodes, cells):
    """Tetrahedron10 / Triangle6 gradient and mass matrices, integrated with
    rules exact for their degrees (gradient products degree 2, function
    products degree 4), as the reference does (core/src/elementmatrix.cpp:
    780-781, 1043-1096; core/src/integration.cpp:302-440)."""
    g, V = _bary_gradients(dim, nodes[cells[:, :dim + 1]])
    if dim == 3:
        a, b = (5.0 + 3.0 * math.sqrt(5.0)) / 20.0, (5.0 - math.sqrt(5.0)) / 20.0
        lam2 = np.full((4, 4), b)
        np.fill_diagonal(lam2, a)
        w2 = np.full(4, 0.25)
        lam4, w4 = _rule_tet_deg4()
    else:
        lam2 = np.array([[0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])
        w2 = np.full(3, 1.0 / 3.0)
        lam4, w4 = _rule_tri_deg4()
    dN = _p2_grad(dim, lam2, g)                               # C x Q x nv x 3
    K = V[:, None, None] * np.einsum("q,cqid,cqjd->cij", w2, dN, dN)
    N = _p2_shape(dim, lam4)                                  # Q x nv
    M = V[:, None, None] * np.einsum("q,qi,qj->ij", w4, N, N)[None]
    return K, M


def element_matrices(dim, nodes, cells):
    """Per-cell gradient matrix K (without 1/rho) and mass matrix M; P2
    cells are handled by element_matrices_p2.  P1 below.

    Triangle K: closed form of elementmatrix.cpp:817-860 with J = 2*area.
    Tetrahedron K: one-point rule, V * grad(N_i) . grad(N_j).
    Mass: A/12 (1 + delta_ij) (triangle), V/20 (1 + delta_ij) (tetrahedron),
    which the reference's quadrature rules integrate exactly."""
    if cells.shape[1] > dim + 1:
        return element_matrices_p2(dim, nodes, cells)
    p = nodes[cells]
    C = len(cells)
    if dim == 2:
        x1, x2, x3 = p[:, 0, 0], p[:, 1, 0], p[:, 2, 0]
        y1, y2, y3 = p[:, 0, 1], p[:, 1, 1], p[:, 2, 1]
        J = np.abs((x2 - x1) * (y3 - y1) - (x3 - x1) * (y2 - y1))
        a = ((x3 - x1) * (x3 - x1) + (y3 - y1) * (y3 - y1)) / J
        b = -((x3 - x1) * (x2 - x1) + (y3 - y1) * (y2 - y1)) / J
        c = ((x2 - x1) * (x2 - x1) + (y2 - y1) * (y2 - y1)) / J
        K = np.empty((C, 3, 3))
        K[:, 0, 0] = a * 0.5 + b + c * 0.5
        K[:, 1, 0] = a * -0.5 + b * -0.5
        K[:, 2, 0] = b * -0.5 + c * -0.5
        K[:, 1, 1] = a * 0.5
        K[:, 2, 1] = b * 0.5
        K[:, 2, 2] = c * 0.5
        K[:, 0, 1] = K[:, 1, 0]
        K[:, 0, 2] = K[:, 2, 0]
        K[:, 1, 2] = K[:, 2, 1]
        area = J / 2.0
        M = (area / 12.0)[:, None, None] * (np.ones((3, 3)) + np.eye(3))[None]
        return K, M
    e1 = p[:, 1] - p[:, 0]
    e2 = p[:, 2] - p[:, 0]
    e3 = p[:, 3] - p[:, 0]
    Jm = np.stack([e1, e2, e3], axis=2)  # columns = edge vectors
    det = np.linalg.det(Jm)
    V = np.abs(det) / 6.0
    inv = np.linalg.inv(Jm)  # rows = grad of barycentric coords 1..3
    G = np.empty((C, 4, 3))
    G[:, 1:, :] = inv
    G[:, 0, :] = -inv.sum(axis=1)
    K = V[:, None, None] * np.einsum("cik,cjk->cij", G, G)
    M = (V / 20.0)[:, None, None] * (np.ones((4, 4)) + np.eye(4))[None]
    return K, M


def boundary_mass(dim, nodes, bnd):
    """u2 of a boundary facet: edge L/6 (1 + delta), triangle A/12 (1 + delta);
    Edge3 L/30 [4 -1 2; -1 4 2; 2 2 16]; Triangle6 with the degree-4 rule."""
    if bnd.shape[1] == 3 and dim == 2:
        L = np.linalg.norm(nodes[bnd[:, 1]] - nodes[bnd[:, 0]], axis=1)
        m = np.array([[4.0, -1.0, 2.0], [-1.0, 4.0, 2.0], [2.0, 2.0, 16.0]])
        return (L / 30.0)[:, None, None] * m[None]
    if bnd.shape[1] == 6:
        p = nodes[bnd[:, :3]]
        A = 0.5 * np.linalg.norm(np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), axis=1)
        lam, w = _rule_tri_deg4()
        N = _p2_shape(2, lam)
        return A[:, None, None] * np.einsum("q,qi,qj->ij", w, N, N)[None]
    p = nodes[bnd]
    if dim == 2:
        L = np.linalg.norm(p[:, 1] - p[:, 0], axis=1)
        return (L / 6.0)[:, None, None] * (np.ones((2, 2)) + np.eye(2))[None]
    A = 0.5 * np.linalg.norm(np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]), axis=1)
    return (A / 12.0)[:, None, None] * (np.ones((3, 3)) + np.eye(3))[None]


def boundary_center_normal(dim, nodes, bnd):
    c = nodes[bnd].mean(axis=1)
    p = nodes[bnd[:, :dim]]
    if dim == 2:
        t = p[:, 1] - p[:, 0]
        n = np.column_stack([t[:, 1], -t[:, 0], np.zeros(len(t))])
    else:
        n = np.cross(p[:, 1] - p[:, 0], p[:, 2] - p[:, 0])
    n = n / np.linalg.norm(n, axis=1)[:, None]
    return c, n


def mixed_bc_alpha(dim, centers, normals, source, k):
    """mixedBoundaryCondition (dcfemmodelling.cpp:430-506), mirror-source
    variant, mirror plane z = 0 on axis dim-1 (y for 2.5-D, z for 3-D)."""
    ax = 2 if k == 0 else 1
    src = np.asarray(source, np.float64)
    mir = src.copy()
    mir[ax] = -src[ax]
    r = src[None, :] - centers
    rm = mir[None, :] - centers
    ra = np.linalg.norm(r, axis=1)
    rma = np.linalg.norm(rm, axis=1)
    rn = np.abs(np.einsum("ij,ij->i", r, normals))
    rmn = np.abs(np.einsum("ij,ij->i", rm, normals))
    if k == 0:
        return ((rma * rma) * rn / ra + (ra * ra) * rmn / rma) / (rma * ra * (ra + rma))
    k0a = besselK0(ra * k)
    k0m = besselK0(rma * k)
    with np.errstate(divide="ignore", invalid="ignore"):
        res = k * (rn / ra * besselK1(ra * k) + rmn / rma * besselK1(rma * k)) / (k0a + k0m)
    res[(np.abs(k0a) < TOLERANCE) | (np.abs(k0m) < TOLERANCE)] = 0.0
    return res


# --------------------------------------------------------------- sparse --
def sparsity_pattern(n, cells):
    """Full symmetric CSR pattern incl. diagonal, rows/cols ascending."""
    nv = cells.shape[1]
    r = np.repeat(cells, nv, axis=1).ravel().astype(np.int64)
    c = np.tile(cells, (1, nv)).ravel().astype(np.int64)
    key = np.unique(r * n + c)
    rows = key // n
    cols = (key % n).astype(np.int32)
    rowptr = np.zeros(n + 1, np.int64)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr).astype(np.int32)
    return rowptr, cols


def find_cell(mesh, p, tol=1e-12):
    """Cell that holds point p (linear triangles / tetrahedra) and the cell's
    shape functions at p (barycentric coordinates): the lowest cell index
    whose coordinates are all >= -tol.  (-1, None) if none."""
    d = mesh.dim()
    if mesh.cells.shape[1] != d + 1:
        raise NotImplementedError("electrodes inside cells need linear cells")
    x = mesh.nodes[mesh.cells][:, :, :d]                       # C x (d+1) x d
    A = np.transpose(x[:, 1:, :] - x[:, :1, :], (0, 2, 1))      # C x d x d
    rhs = p[:d][None, :] - x[:, 0, :]
    lam = np.linalg.solve(A, rhs[:, :, None])[:, :, 0]
    bary = np.column_stack([1.0 - lam.sum(axis=1), lam])
    ok = np.nonzero(np.all(bary >= -tol, axis=1))[0]
    if len(ok) == 0:
        return -1, None
    return int(ok[0]), bary[ok[0]]


class Problem:
    """Mesh + electrodes + scheme with everything that does not depend on the
    resistivity model precomputed."""

    def __init__(self, mesh, sensors, abmn, kfac, k=None, w=None, primary=None, dipole=False):
        """``primary``: unit primary potentials u_p[kIdx, e, node] given (the
        numerical ones of a topographic surface, ``numerical_primary``);
        default the analytic half-space potentials.  ``dipole``: the
        patterns of the dipole current pattern (BoundarySetup): one pure
        pole per electrode, whose differences are the (a, b) dipoles."""
        self.mesh = mesh
        self.dipole = bool(dipole)
        self.dim = mesh.dim()
        nodes = mesh.nodes
        self.n = len(nodes)
        self.abmn = np.asarray(abmn, np.int64).reshape(-1, 4)
        self.kfac = np.asarray(kfac, np.float64)
        self.rowptr, self.cols = sparsity_pattern(self.n, mesh.cells)
        self.K, self.M = element_matrices(self.dim, nodes, mesh.cells)
        self._search_electrodes(np.asarray(sensors, np.float64).reshape(-1, 3))
        if k is None:
            raise ValueError("k/w must be given")
        self.k = np.asarray(k, np.float64)
        self.w = np.asarray(w, np.float64)
        # mixed boundaries
        bm = mesh.boundary_markers
        self.mixed = np.nonzero(bm == -2)[0]
        bnd = mesh.boundaries[self.mixed]
        self.bnd_nodes = bnd
        self.bnd_cell = mesh.boundary_cells[self.mixed]
        self.bnd_mass = boundary_mass(self.dim, nodes, bnd)
        self.bnd_c, self.bnd_n = boundary_center_normal(self.dim, nodes, bnd)
        neu = np.nonzero(bm == -1)[0]
        self._patterns()
        if len(neu):
            cz = boundary_center_normal(self.dim, nodes, mesh.boundaries[neu])[0][:, self.dim - 1]
            self.surfaceZ = float(cz[0])
        else:
            self.surfaceZ = -np.finfo(np.float64).max
        self.alpha = [mixed_bc_alpha(self.dim, self.bnd_c, self.bnd_n, self.src_center, kk)
                      for kk in self.k]
        self._slot_maps()
        if primary is not None:
            self.up = np.asarray(primary, np.float64).reshape(len(self.k), self.nE, self.n).copy()
        else:
            self.up = self._primary()

    # electrode search (dcfemmodelling.cpp:790-1030), node electrodes only
    def _search_electrodes(self, sensors):
        mesh = self.mesh
        ePos = sensors.copy()
        if self.dim == 2:
            zvar = np.ptp(ePos[:, 2]) > 0 or np.max(np.abs(ePos[:, 2])) > 0
            yvar = np.ptp(ePos[:, 1]) > 0
            if zvar and not yvar and np.max(np.abs(ePos[:, 1])) < 1e-8:
                ePos[:, [1, 2]] = ePos[:, [2, 1]]
        cand = list(np.nonzero(mesh.node_markers == -99)[0])
        enodes, epos, erows, ewts, ecell_ent = [], [], [], [], []
        for p in ePos:
            hit = None
            for j, nid in enumerate(cand):
                if np.linalg.norm(p - mesh.nodes[nid]) < 0.01:
                    hit = j
                    break
            if hit is not None:
                nd = cand.pop(hit)
                enodes.append(nd)
                epos.append(mesh.nodes[nd])
                erows.append(np.array([nd]))
                ewts.append(np.ones(1))
                ecell_ent.append(-1)
                continue
            # no electrode node: the cell that holds the sensor (ElectrodeShapeEntity,
            # dcfemmodelling.cpp:924-937, electrode.cpp:252-290)
            cell, wts = find_cell(mesh, p)
            if cell < 0:
                raise ValueError("There is a requested electrode that does not match the given mesh.")
            enodes.append(-1)
            epos.append(p.copy())
            erows.append(mesh.cells[cell].astype(np.int64))
            ewts.append(wts)
            ecell_ent.append(cell)
        self.enodes = np.array(enodes, np.int64)
        self.epos = np.array(epos, np.float64)
        self.erows, self.ewts = erows, ewts
        self.nE = len(self.enodes)
        self.src_center = self.epos.sum(axis=0) / self.nE
        # incident cells and neighbour distance per electrode node (the cell of an entity electrode)
        cells = mesh.cells
        self.ecells = []
        self.eminr = np.zeros(self.nE)
        for i, nd in enumerate(self.enodes):
            if nd < 0:
                self.ecells.append(np.array([ecell_ent[i]]))
                continue
            cs = np.nonzero(np.any(cells == nd, axis=1))[0]
            self.ecells.append(cs)
            nb = np.setdiff1d(np.unique(cells[cs]), [nd])
            self.eminr[i] = np.min(np.linalg.norm(mesh.nodes[nb] - mesh.nodes[nd], axis=1))

    def _patterns(self):
        """Reference electrode and calibration/Dirichlet nodes (BoundarySetup):
        pattern e carries +1 at electrode e and -1 at the reference (sink rows
        and weights; none: the current leaves at infinity)."""
        bc = BoundarySetup(self.mesh, self.nE, getattr(self, "dipole", False))
        self.bc = bc
        self.calib, self.clean = bc.calib, bc.clean
        self.ref_minr, self.ref_cells = 0.0, np.zeros(0, np.int64)
        if bc.ref_node >= 0:
            self.sink = (np.array([bc.ref_node]), np.ones(1))
            self.ref_pos = self.mesh.nodes[bc.ref_node].copy()
            self.ref_minr, self.ref_cells = node_min_radius(self.mesh, bc.ref_node)
        elif bc.ref_elec >= 0:
            r = bc.ref_elec
            self.sink = (self.erows[r], self.ewts[r])
            self.ref_pos = self.epos[r].copy()
        else:
            self.sink = None

    def _slot_maps(self):
        """(cell, i, j) -> CSR slot and (boundary, i, j) -> CSR slot."""
        n = self.n
        key = self.rowptr  # noqa
        rows = np.repeat(np.arange(n), np.diff(self.rowptr))
        fullkey = rows.astype(np.int64) * n + self.cols
        cells = self.mesh.cells.astype(np.int64)
        nv = cells.shape[1]
        ck = cells[:, :, None] * n + cells[:, None, :]
        self.cell_slot = np.searchsorted(fullkey, ck.reshape(len(cells), nv * nv)).reshape(-1, nv, nv)
        b = self.bnd_nodes.astype(np.int64)
        if len(b):
            nb = b.shape[1]
            bk = b[:, :, None] * n + b[:, None, :]
            self.bnd_slot = np.searchsorted(fullkey, bk.reshape(len(b), nb * nb)).reshape(-1, nb, nb)
        else:
            self.bnd_slot = np.zeros((0, self.dim, self.dim), np.int64)

    def _unit_primary(self, src, node, mr, kk):
        """Unit-current half-space potential of a source at src for
        wavenumber kk at every node, with the singular value at its node
        (exactDCSolution + setSingValue)."""
        nodes = self.mesh.nodes
        ax = 1 if kk > 0 else 2
        r = np.linalg.norm(nodes - src, axis=1)
        mir = src.copy()
        mir[ax] = 2.0 * self.surfaceZ - src[ax]
        rm = np.linalg.norm(nodes - mir, axis=1)
        zero = r < TOLERANCE
        rs = np.where(zero, 1.0, r)
        rm = np.where(zero, 1.0, rm)
        if kk == 0.0:
            u = (1.0 / rs + 1.0 / rm) / (4.0 * PI)
        elif np.array_equal(src, mir):
            u = besselK0(rs * kk) / PI
        else:
            u = (besselK0(rs * kk) + besselK0(rm * kk)) / (2.0 * PI)
        u[zero] = 0.0
        if node < 0:
            pass  # entity electrode: no node at the source
        elif kk > 0.0:
            u[node] = besselK0(np.array([mr / 6.0 * kk]))[0] / PI
        else:
            u[node] = 1.0 / (2.0 * PI * mr / 2.0)
        return u

    def _primary(self):
        """u_p[kIdx, e, node] for the unit-current pattern of electrode e
        (exactDCSolution + setSingValue; minus the reference electrode's,
        checkPrimpotentials_, dcfemmodelling.cpp:2085-2090)."""
        up = np.zeros((len(self.k), self.nE, self.n))
        for ki, kk in enumerate(self.k):
            ref = None
            if self.bc.ref_node >= 0:
                ref = self._unit_primary(self.ref_pos, self.bc.ref_node, self.ref_minr, kk)
            elif self.bc.ref_elec >= 0:
                r = self.bc.ref_elec
                ref = self._unit_primary(self.epos[r], self.enodes[r], self.eminr[r], kk)
            for e in range(self.nE):
                up[ki, e] = self._unit_primary(self.epos[e], self.enodes[e], self.eminr[e], kk)
                if ref is not None:
                    up[ki, e] -= ref
        return up

    # ---------------------------------------------------------- assembly --
    def assemble(self, rho_cell, kidx):
        """System matrix values (CSR order) for wavenumber index kidx."""
        kk = self.k[kidx]
        vals = np.zeros(len(self.cols))
        Se = self.M * (kk * kk) + self.K if kk > 0.0 else self.K
        valid = np.abs(rho_cell) > TOLERANCE
        contrib = Se * (1.0 / np.where(valid, rho_cell, 1.0))[:, None, None]
        contrib[~valid] = 0.0
        np.add.at(vals, self.cell_slot.ravel(), contrib.ravel())
        # forced homogeneous Dirichlet where the diagonal vanished
        diag_slot = self._diag_slots()
        bad = np.nonzero(vals[diag_slot] < TOLERANCE)[0]
        if len(bad):
            self._clean_rows_cols(vals, bad, diag_slot)
        if len(self.mixed):
            rb = rho_cell[self.bnd_cell]
            bc = self.bnd_mass * (self.alpha[kidx] / rb)[:, None, None]
            np.add.at(vals, self.bnd_slot.ravel(), bc.ravel())
        if len(self.clean):  # homogeneous Dirichlet boundaries, then calibration nodes
            self._clean_rows_cols(vals, self.clean, diag_slot)
        return vals

    def _diag_slots(self):
        rows = np.arange(self.n)
        rk = np.repeat(np.arange(self.n), np.diff(self.rowptr)).astype(np.int64) * self.n + self.cols
        return np.searchsorted(rk, rows.astype(np.int64) * self.n + rows)

    def _clean_rows_cols(self, vals, nodes_, diag_slot):
        rows = np.repeat(np.arange(self.n), np.diff(self.rowptr))
        kill = np.isin(rows, nodes_) | np.isin(self.cols, nodes_)
        vals[kill] = 0.0
        vals[diag_slot[nodes_]] = 1.0

    def csr(self, vals):
        return sp.csr_matrix((vals, self.cols, self.rowptr), shape=(self.n, self.n))

    # ---------------------------------------------------------- forward --
    def source_rho(self, rho_cell):
        """Source resistivity of each electrode's pattern: the geometric mean
        of the cells around the electrode node, averaged with the reference
        electrode's over those above TOLERANCE (calculateK,
        dcfemmodelling.cpp:2236-2266)."""
        gm = np.array([np.exp(np.mean(np.log(rho_cell[c]))) for c in self.ecells])
        if self.sink is None:
            return gm
        if self.bc.ref_node >= 0:
            rr = float(np.exp(np.mean(np.log(rho_cell[self.ref_cells]))))
        else:
            rr = float(gm[self.bc.ref_elec])
        out = np.empty_like(gm)
        for e, ra in enumerate(gm):
            v = [x for x in (ra, rr) if x > TOLERANCE]
            out[e] = sum(v) / len(v)
        return out

    def solve(self, rho_cell):
        """Sub-potentials u[kIdx, e, node] (SR total potentials per k)."""
        nK = len(self.k)
        u = np.zeros((nK, self.nE, self.n))
        rs = self.source_rho(rho_cell)
        ones = np.ones_like(rho_cell)
        for ki in range(nK):
            S = self.csr(self.assemble(rho_cell, ki))
            S1 = self.csr(self.assemble(ones, ki))
            lu = spla.splu(S.tocsc(), permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0)
            for e in range(self.nE):
                prim = self.up[ki, e] * rs[e]
                rhs = S1 @ prim / rs[e] - S @ prim
                rhs[self.calib] = 0.0
                u[ki, e] = lu.solve(rhs) + prim
        return u

    def collect(self, u):
        """Electrode potential matrix U[e, f] = sum_k w_k u_k[e](node f)."""
        sol = np.einsum("k,ken->en", self.w, u)
        return np.stack([sol[:, r] @ w for r, w in zip(self.erows, self.ewts)], axis=1)

    def data_u(self, U, reciprocity=False):
        ab = self.abmn
        a, b, m, n = ab[:, 0], ab[:, 1], ab[:, 2], ab[:, 3]
        if reciprocity:
            a, m = m, a
            b, n = n, b

        def g(i, j):
            ok = (i != -1) & (j != -1)
            return np.where(ok, U[np.where(ok, i, 0), np.where(ok, j, 0)], 0.0)

        uAM, uAN, uBM, uBN = g(a, m), g(a, n), g(b, m), g(b, n)
        return (uAM - uAN) - (uBM - uBN)

    def calculate(self, rho_cell):
        """Signed voltages of the data for a unit current, without rounding
        or reciprocity (DCMultiElectrodeModelling::calculate(DataContainerERT
        &), dcfemmodelling.cpp:1558-1618); with ``dipole`` the voltage of an
        (a, b) pattern is the difference of the pure poles a and b."""
        return Problem.data_u(self, self.collect(self.solve(rho_cell)))

    def response_from_u(self, u):
        U = self.collect(u)
        r = np.rint(self.data_u(U) / 1e-10) * 1e-10
        rr = np.rint(self.data_u(U, True) / 1e-10) * 1e-10
        r = r * self.kfac
        rr = rr * self.kfac
        return np.sqrt(np.abs(r * rr))

    def response(self, rho_cell):
        if np.min(rho_cell) < TOLERANCE:
            raise ValueError("response for model with negative or zero resistivity is not defined")
        u = self.solve(rho_cell)
        return self.response_from_u(u), u

    # --------------------------------------------------------- Jacobian --
    def jacobian(self, u, model, n_params=None):
        """J[d, p] (bertJacobian.cpp calc2 + dcfemmodelling.cpp:1377-1384)."""
        mk = self.mesh.cell_markers
        P = int(mk.max()) + 1 if n_params is None else n_params
        D = len(self.abmn)
        J = np.zeros((D, P))
        cells = self.mesh.cells
        sel = np.nonzero(mk >= 0)[0]
        ab = self.abmn
        for ki, kk in enumerate(self.k):
            S = self.M[sel] * (kk * kk) + self.K[sel]
            Uc = np.transpose(u[ki][:, cells[sel]], (1, 2, 0))  # C x nv x nE
            Uc = np.concatenate([Uc, np.zeros(Uc.shape[:2] + (1,))], axis=2)  # index -1 -> 0
            V = np.einsum("cij,cje->cie", S, Uc)
            a, b, m, n = ab[:, 0], ab[:, 1], ab[:, 2], ab[:, 3]
            dab = V[:, :, a] - V[:, :, b]          # C x nv x D
            dmn = Uc[:, :, m] - Uc[:, :, n]
            contrib = np.einsum("cid,cid->dc", dab, dmn) * self.w[ki]
            np.add.at(J.T, mk[sel], contrib.T)
        if len(model) == P:
            J = J / ((np.asarray(model) ** 2)[None, :] / self.kfac[:, None])
        return J

    # ------------------------------------------------ complex resistivity --
    # With complex resistivities the reference's SR operator falls back to
    # the total-potential formulation of DCMultiElectrodeModelling
    # (calculateK_, core/src/bert/dcfemmodelling.cpp:1756-1929): complex
    # symmetric matrices sum (1/rho*) (K + k^2 M) + mixed term alpha / rho*,
    # a unit point source at the current electrode's node, no singularity
    # removal, no rounding and no reciprocity in the response.
    def assemble_complex(self, rho_c, kidx):
        """Complex system matrix values (CSR order) for wavenumber kidx
        (dcfemmodelling.cpp:163-215, 217-300 with complex attributes)."""
        kk = self.k[kidx]
        vals = np.zeros(len(self.cols), complex)
        Se = self.M * (kk * kk) + self.K if kk > 0.0 else self.K
        rho_c = np.asarray(rho_c, complex)
        valid = np.abs(rho_c) > TOLERANCE
        sigma = np.where(valid, 1.0 / np.where(valid, rho_c, 1.0), 0.0)
        np.add.at(vals, self.cell_slot.ravel(), (Se * sigma[:, None, None]).ravel())
        if len(self.mixed):
            bc = self.bnd_mass * (self.alpha[kidx] / rho_c[self.bnd_cell])[:, None, None]
            np.add.at(vals, self.bnd_slot.ravel(), bc.ravel())
        return vals

    def solve_complex(self, rho_c):
        """Total potentials u[kIdx, e, node] for a unit source at each
        electrode node (ElectrodeShapeNode::assembleRHS, electrode.cpp:133-141)."""
        nK = len(self.k)
        u = np.zeros((nK, self.nE, self.n), complex)
        for ki in range(nK):
            S = sp.csr_matrix((self.assemble_complex(rho_c, ki), self.cols, self.rowptr), shape=(self.n, self.n))
            lu = spla.splu(S.tocsc(), permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0)
            for e in range(self.nE):
                rhs = np.zeros(self.n, complex)
                rhs[self.erows[e]] = self.ewts[e]
                u[ki, e] = lu.solve(rhs)
        return u

    def response_complex(self, rho_c):
        """Complex apparent resistivities k * u_ABMN (dcfemmodelling.cpp:
        1103-1119, DataMap::data, datamap.cpp:159-232) and the potentials."""
        rho_c = np.asarray(rho_c, complex)
        if np.min(np.abs(rho_c)) < TOLERANCE:
            raise ValueError("complex response for abs model with negative or zero resistivity is not defined")
        u = self.solve_complex(rho_c)
        return self.data_u(self.collect(u)) * self.kfac, u

    def jacobian_complex(self, u, model_c, n_params=None):
        """Complex J[d, p] (createSensitivityCol with complex potentials,
        J /= model^2 / k without conjugation, dcfemmodelling.cpp:1410-1431)."""
        mk = self.mesh.cell_markers
        P = int(mk.max()) + 1 if n_params is None else n_params
        J = np.zeros((len(self.abmn), P), complex)
        cells = self.mesh.cells
        sel = np.nonzero(mk >= 0)[0]
        ab = self.abmn
        for ki, kk in enumerate(self.k):
            S = self.M[sel] * (kk * kk) + self.K[sel]
            Uc = np.transpose(u[ki][:, cells[sel]], (1, 2, 0))
            Uc = np.concatenate([Uc, np.zeros(Uc.shape[:2] + (1,), complex)], axis=2)
            V = np.einsum("cij,cje->cie", S, Uc)
            a, b, m, n = ab[:, 0], ab[:, 1], ab[:, 2], ab[:, 3]
            contrib = np.einsum("cid,cid->dc", V[:, :, a] - V[:, :, b], Uc[:, :, m] - Uc[:, :, n]) * self.w[ki]
            np.add.at(J.T, mk[sel], contrib.T)
        model_c = np.asarray(model_c, complex)
        if len(model_c) == P:
            J = J / ((model_c ** 2)[None, :] / self.kfac[:, None])
        return J


def map_model(mesh, model, background=-9e99):
    """createMappedModel (modellingbase.cpp:401-497) without fixed regions:
    model[marker] per cell; marker -1 cells prolongated from neighbours."""
    model = np.asarray(model, np.float64)
    mk = mesh.cell_markers
    C = mesh.cellCount()
    if len(model) == C:
        if len(np.unique(mk[mk > -1])) != len(model):
            return model.copy()
    att = np.zeros(C)
    pos = mk >= 0
    if np.any(mk[pos] >= len(model)):
        raise ValueError("marker >= model size")
    att[pos] = model[mk[pos]]
    if background != 0.0:
        prolongate_empty(mesh, att, background)
    return att


def prolongate_empty(mesh, vals, background):
    """Mesh::prolongateEmptyCellsValues (mesh.cpp:2247-2316)."""
    empty = np.nonzero(np.abs(vals) < TOLERANCE)[0]
    if len(empty) == 0:
        return
    if background > -9e99:
        vals[empty] = background
        return
    cells = mesh.cells
    nv = cells.shape[1]
    # neighbour cells through shared facets
    faces, owner = [], []
    for skip in range(nv):
        cols = [j for j in range(nv) if j != skip]
        faces.append(np.sort(cells[:, cols], axis=1))
        owner.append(np.arange(len(cells)))
    faces = np.concatenate(faces)
    owner = np.concatenate(owner)
    key = faces[:, 0].astype(np.int64)
    for j in range(1, faces.shape[1]):
        key = key * mesh.nodeCount() + faces[:, j]
    order = np.argsort(key, kind="stable")
    key, owner, faces = key[order], owner[order], faces[order]
    nbr = {}
    same = np.nonzero(key[1:] == key[:-1])[0]
    for i in same:
        c1, c2 = owner[i], owner[i + 1]
        nbr.setdefault(c1, []).append((c2, faces[i]))
        nbr.setdefault(c2, []).append((c1, faces[i]))
    XY = np.array([1.0, 1.0, 0.0])
    if mesh.dim() == 2:
        XY[1] = 0.0
    from oracle.ert_oracle import boundary_center_normal  # noqa: self import for clarity
    while True:
        empty = np.nonzero(np.abs(vals) < TOLERANCE)[0]
        if len(empty) == 0:
            return
        upd = {}
        for c in empty:
            wsum = 0.0
            vsum = 0.0
            for (nc, f) in nbr.get(c, []):
                if abs(vals[nc]) > TOLERANCE:
                    nrm = boundary_center_normal(mesh.dim(), mesh.nodes, f[None, :])[1][0]
                    zw = np.linalg.norm(nrm * XY) + 1e-6
                    vsum += vals[nc] * zw
                    wsum += zw
            if wsum > 1e-8:
                upd[c] = vsum / wsum
        if not upd:
            raise ValueError("cannot prolongate empty cells")
        for c, v in upd.items():
            vals[c] = v


def numerical_primary(mesh, sensors, abmn, kfac, k, w, dipole=False):
    """Unit primary potentials of a topographic surface
    (DCSRMultiElectrodeModelling::checkPrimpotentials_,
    core/src/bert/dcfemmodelling.cpp:2008-2068): the total potential at 1
    Ohm m on createP2 of the mesh (cem_oracle.TotalPotentialProblem, direct
    solve), taken at the mesh's own nodes (createP2 keeps them first; the
    reference's interpolation to a vertex is its nodal value).
    Returns u_p[kIdx, e, node]."""
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    if here not in sys.path:
        sys.path.insert(0, here)
    from cem_oracle import TotalPotentialProblem
    m2 = mesh.createP2()
    T = TotalPotentialProblem(m2, sensors, abmn, kfac, k, w, dipole=dipole)
    u = T.solve(np.ones(m2.cellCount()))
    return u[:, :, :mesh.nodeCount()].copy()
