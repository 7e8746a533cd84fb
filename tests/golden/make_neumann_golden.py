"""Generate the fixtures of closed (Neumann-only) domains, reference and
calibration nodes and homogeneous Dirichlet boundaries from the reference's
own C++ (oracle/_ref/libgimli_ref.so, built by ``make -C oracle``) through
oracle/ref_driver.py:

    python tests/golden/make_neumann_golden.py [fixture names ...]

The reference (core/src/bert/dcfemmodelling.cpp):

* a mesh with no mixed (-2) and no Dirichlet (-3, -4) boundary is a Neumann
  domain (updateMeshDependency_, 711-773); it counts as topography (primary
  potentials and geometric factors numerical), and in 3-D the potential is
  fixed at calibration nodes (node marker -1000, else node 0: homogeneous
  Dirichlet rows, 2182-2192, zero singularity-removal right-hand side there,
  2281-2283) and the current flows from each electrode to a reference
  electrode (node marker -999, else the last electrode, whose own pattern is
  then left out: searchElectrodes_ 1011-1073, createCurrentPattern
  1515-1523, DataMap::data core/src/bert/datamap.cpp:203-214);
* a reference-electrode node also gives (electrode, reference) patterns in a
  domain with mixed boundaries (searchElectrodes_ 1011-1015);
* homogeneous Dirichlet boundaries (-3) clean their nodes' rows and columns
  (dcfemBoundaryAssembleStiffnessMatrix 279-298).

With the reference at the last electrode (no reference node) the reference's
createJacobian stops with "potential matrix rowsize to small" (its
potentials have one row less than electrodes, core/src/bert/
bertJacobian.cpp:285-290); those fixtures hold central differences of the
reference's own response for a few parameters instead (``fd_params``,
``fd_J``: d rhoa / d rho, relative step 1e-4).

The singularity-removal fixtures of Neumann domains take their primary
potentials the way make_sr_topo_golden.py does (the reference's
total-potential operator at 1 Ohm m on createP2, given with
setPrimaryPotential): the reference's own internal solve has no
factorization in this build.

Fixtures (inputs, k/w, the factored system matrix of the first wavenumber,
sub-potentials of the first wavenumber, apparent resistivities, Jacobian or
its finite differences):

  ert3d_neumann_tp_small      closed 3-D box, no markers (calibration node 0,
  ert3d_neumann_sr_small      reference at the last electrode)
  ert3d_neumann_ref_tp_small  closed 3-D box with a reference node (-999) and
  ert3d_neumann_ref_sr_small  a calibration node (-1000)
  ert3d_refnode_sr_small      3-D box with mixed boundaries and a reference
  ert3d_refnode_tp_small      node (analytic primaries minus the reference's)
  ert3d_dirichlet_sr_small    3-D box: bottom homogeneous Dirichlet (-3),
  ert3d_dirichlet_tp_small    sides mixed
  ert2d_neumann_sr_small      2-D mesh with Neumann boundaries only (2.5-D:
  ert2d_neumann_tp_small      topography, no calibration, no reference)

Run from the repository root.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from make_cem_golden import _resistivity  # noqa: E402
from oracle.ref_driver import RefModelling  # noqa: E402
from pygimli_gb300.data import DataContainerERT, createData, geometricFactors  # noqa: E402
from pygimli_gb300.mesh import Mesh, create_box_mesh_3d, create_para_mesh_2d  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
only = set(sys.argv[1:])
FD_PARAMS = 6


def _numerical_primary(mesh, data):
    """Total potential at 1 Ohm m on createP2 of the mesh, at the mesh's nodes."""
    T = RefModelling(mesh, data.sensorPositions(), data.abmn(), np.ones(data.size()), sr=False, p2=True)
    k, w = T.kw()
    T.response(np.ones(T.mesh_arrays()[2].shape[0]))
    prim = T.subpotentials()[:, :mesh.nodeCount()].copy()
    T.close()
    return prim, k, w


def case(name, mesh, data, seed, sr, numerical=False, jacobian=True):
    if only and name not in only:
        return
    prim = None
    if sr and numerical:
        prim, k, w = _numerical_primary(mesh, data)
    R = RefModelling(mesh, data.sensorPositions(), data.abmn(), data["k"], sr=sr, keep_matrices=True)
    if prim is not None:
        R.set_kw(k, w)
        R.set_primary(prim)
    k, w = R.kw()
    rho = _resistivity(mesh, seed)
    rhoa = R.response(rho)
    rp, ci, va = R.matrices[0]
    sub = R.subpotentials()
    npat = sub.shape[0] // len(k)
    sub = sub.reshape(len(k), npat, -1)
    extra = {}
    if jacobian:
        extra["J"] = R.jacobian(rho)
    else:
        rng = np.random.default_rng(seed + 1000)
        params = np.sort(rng.choice(mesh.cellCount(), FD_PARAMS, replace=False))
        fd = np.zeros((data.size(), len(params)))
        for j, p in enumerate(params):
            h = 1e-4 * rho[p]
            rp_, rm_ = rho.copy(), rho.copy()
            rp_[p] += h
            rm_[p] -= h
            fd[:, j] = (R.response(rp_) - R.response(rm_)) / (2.0 * h)
        extra["fd_params"] = params
        extra["fd_J"] = fd
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"), **extra,
        dim=mesh.dim(), nodes=mesh.nodes, cells=mesh.cells, cell_markers=mesh.cell_markers,
        node_markers=mesh.node_markers, boundaries=mesh.boundaries,
        boundary_markers=mesh.boundary_markers, boundary_cells=mesh.boundary_cells,
        sensors=data.sensorPositions(), abmn=data.abmn(), kfac=data["k"], k=k, w=w, rho=rho, rhoa=rhoa,
        rowptr=rp, colidx=ci, S=va, subpot=sub[0], sr=int(bool(sr)),
        primary=np.zeros(0) if prim is None else prim.reshape(len(k), npat, -1)[0],
        electrode_nodes=R.electrode_nodes())
    R.close()
    print(name, mesh, len(data), "k:", len(k), "patterns:", npat, "J:" if jacobian else "fd:",
          extra["J"].shape if jacobian else extra["fd_J"].shape)


def _remark(m, bm=None, nm=None):
    return Mesh(m.dim(), m.nodes, m.cells, m.cell_markers, m.node_markers if nm is None else nm, m.boundaries,
                m.boundary_markers if bm is None else bm, m.boundary_cells, check=False)


def _nearest(m, p):
    return int(np.argmin(np.linalg.norm(m.nodes - np.asarray(p, float), axis=1)))


def main():
    e = np.array([(x, y) for x in (0.0, 2.0, 4.0) for y in (0.0, 2.0)], float)
    m3 = create_box_mesh_3d(e, h=1.0, para_margin=(1, 1), para_depth=3.0, outer=12.0, growth=2.0,
                            depth_growth=1.5)
    ab = np.array([[0, 1, 2, 3], [0, 2, 4, 5], [1, 3, 4, 5], [5, 0, 1, 2], [2, 5, 0, 1], [0, -1, 5, 3],
                   [3, 4, 1, 0], [4, 1, 3, 2]], np.int32)
    d3 = DataContainerERT(np.column_stack([e, np.zeros(len(e))]), ab)
    d3["k"] = geometricFactors(d3, 3)
    # closed box: every boundary homogeneous Neumann
    closed = _remark(m3, bm=np.full(len(m3.boundary_markers), -1, np.int32))
    case("ert3d_neumann_tp_small", closed, d3, seed=41, sr=False, jacobian=False)
    case("ert3d_neumann_sr_small", closed, d3, seed=42, sr=True, numerical=True, jacobian=False)
    # reference node deep below the electrodes, calibration node at a far bottom corner
    nm = closed.node_markers.copy()
    ref = _nearest(closed, (2.0, 1.0, -3.0))
    cal = _nearest(closed, (closed.nodes[:, 0].min(), closed.nodes[:, 1].min(), closed.nodes[:, 2].min()))
    assert nm[ref] == 0 and nm[cal] == 0 and ref != cal
    nm[ref] = -999
    nm[cal] = -1000
    closed_ref = _remark(closed, nm=nm)
    case("ert3d_neumann_ref_tp_small", closed_ref, d3, seed=43, sr=False)
    case("ert3d_neumann_ref_sr_small", closed_ref, d3, seed=44, sr=True, numerical=True)
    # mixed boundaries and a reference node
    nm2 = m3.node_markers.copy()
    nm2[ref] = -999
    refnode = _remark(m3, nm=nm2)
    case("ert3d_refnode_sr_small", refnode, d3, seed=45, sr=True)
    case("ert3d_refnode_tp_small", refnode, d3, seed=46, sr=False)
    # bottom homogeneous Dirichlet, sides mixed
    zc = m3.nodes[m3.boundaries].mean(axis=1)[:, 2]
    bm = m3.boundary_markers.copy()
    bm[np.abs(zc - m3.nodes[:, 2].min()) < 1e-9] = -3
    assert np.any(bm == -3) and np.any(bm == -2)
    dirich = _remark(m3, bm=bm)
    case("ert3d_dirichlet_sr_small", dirich, d3, seed=47, sr=True)
    case("ert3d_dirichlet_tp_small", dirich, d3, seed=48, sr=False)
    # 2-D: Neumann boundaries only (topography for the reference, 2.5-D keeps no calibration)
    xs = np.arange(7.0)
    m2 = create_para_mesh_2d(xs, para_dx=0.25, para_depth=3.0)
    m2n = _remark(m2, bm=np.full(len(m2.boundary_markers), -1, np.int32))
    d2 = createData(xs, "dd")
    d2["k"] = geometricFactors(d2, 2)
    case("ert2d_neumann_sr_small", m2n, d2, seed=49, sr=True, numerical=True)
    case("ert2d_neumann_tp_small", m2n, d2, seed=50, sr=False)


if __name__ == "__main__":
    main()
