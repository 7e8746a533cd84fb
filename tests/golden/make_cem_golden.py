"""Generate the fixtures of the total-potential operator (pyGIMLi
ERTModelling(sr=False), the reference's DCMultiElectrodeModelling) by running
the reference's own C++ (oracle/_ref/libgimli_ref.so, built by
``make -C oracle``) through oracle/ref_driver.py:

    python tests/golden/make_cem_golden.py [fixture names ...]

Fixtures (inputs, reference k/w, the reference's assembled system matrix of
the first wavenumber, the node sub-potentials of the first and the last
wavenumber, apparent resistivities and the Jacobian):

  ert2d_tp_small      2.5-D, 7 node electrodes, dipole-dipole
  ert2d_cem_small     2.5-D, 7 CEM electrodes (two surface edges each,
                      contact impedances 0.5-2 Ohm m^2) and one passive body
  ert3d_cem_small     3-D, 2 x 2 CEM electrodes (2 x 2 m surface patches)
                      beside 2 node electrodes
  ert2d_cem_p2_small  ert2d_cem_small and
  ert3d_cem_p2_small  ert3d_cem_small on the reference's createP2 of the mesh
                      (the 3-D one without the assembled matrix: size)
  ert2d_bypass_small  2.5-D, electrodes 2 and 5 as bypass electrodes (four
                      nodes down from the surface, default 1e-6 Ohm)
  ert2d_topo_tp_small 2.5-D node electrodes on a sinusoidal surface; also the
  ert3d_topo_tp_small 3-D likewise; both also hold the reference's k-summed
                      electrode potential matrices for the model (U) and for
                      1 Ohm m (U1)

Run from the repository root; the working directory must hold none of the
reference's map files (bypass.map, contactImpedance.map, ...).
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.ref_driver import RefModelling  # noqa: E402
from pygimli_gb300.cem import MARKER_BOUND_ELECTRODE, mark_cem_electrodes  # noqa: E402
from pygimli_gb300.data import DataContainerERT, createData, geometricFactors  # noqa: E402
from pygimli_gb300.mesh import Mesh, create_box_mesh_3d, create_para_mesh_2d  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
only = set(sys.argv[1:])


def _resistivity(mesh, seed):
    rng = np.random.default_rng(seed)
    return np.exp(rng.uniform(np.log(50.0), np.log(200.0), mesh.cellCount()))


def _electrode_potentials(R, k, w, nE):
    """The reference's k-summed electrode potential matrix (solutions_ at
    the electrode nodes, dcfemmodelling.cpp:1707-1729, DataMap::collect)."""
    sub = R.subpotentials().reshape(len(k), nE, -1)
    sol = sub[0] * w[0]
    for ki in range(1, len(k)):
        sol += sub[ki] * w[ki]
    return sol[:, R.electrode_nodes()]


def case(name, mesh, data, seed, contact_impedance=None, potentials=False, p2=False, matrix=True):
    """One fixture; with p2 the reference refines the mesh itself
    (Mesh::createP2) and the resistivity is one value per refined cell;
    matrix=False leaves the assembled matrix out (size)."""
    if only and name not in only:
        return
    for f in ("bypass.map", "electrodeBypassResistances.map", "contactImpedance.map", "contactResistance.map"):
        if os.path.exists(f):
            raise SystemExit(f"{f} in the working directory would change the reference's result")
    R = RefModelling(mesh, data.sensorPositions(), data.abmn(), data["k"], keep_matrices=True, sr=False,
                     contact_impedance=contact_impedance, p2=p2)
    k, w = R.kw()
    rho = _resistivity(mesh, seed)
    rhoa = R.response(rho)
    rp, ci, va = R.matrices[0] if matrix else (np.zeros(0, np.int32), np.zeros(0, np.int32), np.zeros(0))
    sub = R.subpotentials().reshape(len(k), data.sensorCount(), -1)
    J = R.jacobian(rho)
    extra = {}
    if potentials:  # node electrodes only: U for the model and for 1 Ohm m
        extra["U"] = _electrode_potentials(R, k, w, data.sensorCount())
        R.response(np.ones(mesh.cellCount()))
        extra["U1"] = _electrode_potentials(R, k, w, data.sensorCount())
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"), **extra,
        dim=mesh.dim(), nodes=mesh.nodes, cells=mesh.cells, cell_markers=mesh.cell_markers,
        node_markers=mesh.node_markers, boundaries=mesh.boundaries,
        boundary_markers=mesh.boundary_markers, boundary_cells=mesh.boundary_cells,
        sensors=data.sensorPositions(), abmn=data.abmn(), kfac=data["k"], k=k, w=w, rho=rho, rhoa=rhoa,
        rowptr=rp, colidx=ci, S=va, subpot_first=sub[0], subpot_last=sub[-1] if len(k) > 1 else np.zeros(0), J=J,
        contact_impedance=np.zeros(0) if contact_impedance is None else np.asarray(contact_impedance, float),
        p2=int(bool(p2)))
    R.close()
    print(name, mesh, len(data), "k:", len(k), "matrix rows:", max(len(rp) - 1, 0), "J:", J.shape)


def main():
    xs = np.arange(7.0)
    m2 = create_para_mesh_2d(xs, para_dx=0.25, para_depth=3.0)
    d2 = createData(xs, "dd")
    d2["k"] = geometricFactors(d2, 2)
    case("ert2d_tp_small", m2, d2, seed=21)
    # CEM: two surface edges per electrode, a passive body between 3 and 4
    m2c = mark_cem_electrodes(m2, np.column_stack([xs, np.zeros_like(xs)]), 0.25, passive=[((3.5, 0.0), 0.25)])
    zc = np.random.default_rng(22).uniform(0.5, 2.0, len(xs) + 1)
    case("ert2d_cem_small", m2c, d2, seed=23, contact_impedance=zc)
    # 3-D: four CEM patches (every surface triangle within 1.42 m) and two node electrodes
    e = np.array([(x, y) for x in (0.0, 4.0) for y in (0.0, 4.0)] + [(2.0, 0.0), (2.0, 4.0)])
    m3 = create_box_mesh_3d(e, h=1.0, para_margin=(1, 1), para_depth=3.0, outer=30.0, growth=2.0, depth_growth=1.5)
    m3c = mark_cem_electrodes(m3, e[:4], 1.42)
    nm = m3c.node_markers.copy()
    for p in e[4:]:
        nd = np.nonzero(np.linalg.norm(m3c.nodes - np.array([p[0], p[1], 0.0]), axis=1) < 1e-9)[0]
        nm[nd] = -99
    m3c = Mesh(3, m3c.nodes, m3c.cells, m3c.cell_markers, nm, m3c.boundaries, m3c.boundary_markers,
               m3c.boundary_cells, check=False)
    ab3 = np.array([[0, 1, 2, 3], [0, 2, 1, 3], [0, 4, 1, 5], [4, 5, 0, 3], [1, 3, 4, 2], [0, 3, 4, 5],
                    [2, 3, 0, 4], [5, 2, 1, 0]], np.int32)
    d3 = DataContainerERT(np.column_stack([e, np.zeros(len(e))]), ab3)
    d3["k"] = geometricFactors(d3, 3)
    case("ert3d_cem_small", m3c, d3, seed=24)
    # quadratic elements: CEM on Edge3 / Triangle6 boundaries
    case("ert2d_cem_p2_small", m2c, d2, seed=28, contact_impedance=zc, p2=True)
    case("ert3d_cem_p2_small", m3c, d3, seed=29, p2=True, matrix=False)
    # bypass electrodes: the surface node and the three below it
    nmb = m2.node_markers.copy()
    for i in (2, 5):
        col = np.nonzero((np.abs(m2.nodes[:, 0] - xs[i]) < 1e-9) & (m2.nodes[:, 1] >= -1.0))[0]
        nmb[col] = MARKER_BOUND_ELECTRODE - i
    m2b = Mesh(2, m2.nodes, m2.cells, m2.cell_markers, nmb, m2.boundaries, m2.boundary_markers, m2.boundary_cells,
               check=False)
    case("ert2d_bypass_small", m2b, d2, seed=25)
    # topography (total potential only): a smooth surface, electrodes on it
    case("ert2d_topo_tp_small", *_topo_2d(m2, xs), seed=26, potentials=True)
    m3n = Mesh(3, m3.nodes, m3.cells, m3.cell_markers, m3.node_markers, m3.boundaries, m3.boundary_markers,
               m3.boundary_cells, check=False)
    case("ert3d_topo_tp_small", *_topo_3d(m3n, e, ab3), seed=27, potentials=True)


def _bend(nodes, axis, t):
    """Raise the surface (coordinate 0 on ``axis``) by t(x[, y]), fading
    linearly to zero at the bottom of the mesh."""
    out = nodes.copy()
    H = -nodes[:, axis].min()
    out[:, axis] = nodes[:, axis] + t * (1.0 + nodes[:, axis] / H)
    return out


def _topo_2d(m, xs):
    t = 0.4 * np.sin(2.0 * np.pi * m.nodes[:, 0] / 6.0)
    mt = Mesh(2, _bend(m.nodes, 1, t), m.cells, m.cell_markers, m.node_markers, m.boundaries, m.boundary_markers,
              m.boundary_cells, check=False)
    en = [int(np.nonzero((np.abs(m.nodes[:, 0] - x) < 1e-9) & (m.node_markers == -99))[0][0]) for x in xs]
    d = DataContainerERT(mt.nodes[en], createData(xs, "dd").abmn())
    d["k"] = geometricFactors(d, 2)
    return mt, d


def _topo_3d(m, e, ab):
    t = 0.3 * np.sin(2.0 * np.pi * m.nodes[:, 0] / 8.0) * np.cos(2.0 * np.pi * m.nodes[:, 1] / 10.0)
    mt = Mesh(3, _bend(m.nodes, 2, t), m.cells, m.cell_markers, m.node_markers, m.boundaries, m.boundary_markers,
              m.boundary_cells, check=False)
    en = [int(np.nonzero(np.linalg.norm(m.nodes[:, :2] - p, axis=1) + np.abs(m.nodes[:, 2]) < 1e-9)[0][0]) for p in e]
    d = DataContainerERT(mt.nodes[en], ab)
    d["k"] = geometricFactors(d, 3)
    return mt, d


if __name__ == "__main__":
    main()
