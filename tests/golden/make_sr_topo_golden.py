"""Generate the fixtures of singularity removal on a topographic surface
(pyGIMLi ERTModelling(), the reference's DCSRMultiElectrodeModelling) from
the reference's own C++ (oracle/_ref/libgimli_ref.so, built by
``make -C oracle``) through oracle/ref_driver.py:

    python tests/golden/make_sr_topo_golden.py [fixture names ...]

On a surface that is not flat the reference computes the primary potentials
numerically (DCSRMultiElectrodeModelling::checkPrimpotentials_,
core/src/bert/dcfemmodelling.cpp:1986-2141): its total-potential operator
DCMultiElectrodeModelling at 1 Ohm m on Mesh::createP2 of the mesh, the
sub-potentials interpolated to the mesh's nodes.  Its internal solve uses the
default LinSolver, which has no factorization without CHOLMOD, so the steps
run here one by one with the reference's own code and the oracle's direct
solve: createP2 and the total-potential operator at 1 Ohm m (primary
sub-potentials), their values at the original nodes (createP2 keeps them
first; the interpolation at a vertex is its nodal value), given to the
singularity-removal operator with setPrimaryPotential
(dcfemmodelling.h:374); then its response and Jacobian.

Fixtures (inputs, k/w, the primary potentials of the first wavenumber, the
singularity-removal sub-potentials of the first wavenumber, apparent
resistivities, Jacobian):

  ert2d_topo_sr_small  2.5-D, 7 node electrodes on a sinusoidal surface
  ert3d_topo_sr_small  3-D, 6 node electrodes on a sinusoidal surface

Run from the repository root.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from make_cem_golden import _resistivity, _topo_2d, _topo_3d  # noqa: E402
from oracle.ref_driver import RefModelling  # noqa: E402
from pygimli_gb300.mesh import Mesh, create_box_mesh_3d, create_para_mesh_2d  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
only = set(sys.argv[1:])


def case(name, mesh, data, seed):
    if only and name not in only:
        return
    n = mesh.nodeCount()
    # primary potentials: total potential at 1 Ohm m on createP2 of the mesh
    T = RefModelling(mesh, data.sensorPositions(), data.abmn(), data["k"], sr=False, p2=True)
    k, w = T.kw()
    T.response(np.ones(T.mesh_arrays()[2].shape[0]))
    prim = T.subpotentials()[:, :n].copy()  # rows = source + k * nE
    T.close()
    R = RefModelling(mesh, data.sensorPositions(), data.abmn(), data["k"], sr=True)
    R.set_kw(k, w)
    R.set_primary(prim)
    rho = _resistivity(mesh, seed)
    rhoa = R.response(rho)
    sub = R.subpotentials().reshape(len(k), data.sensorCount(), -1)
    J = R.jacobian(rho)
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"),
        dim=mesh.dim(), nodes=mesh.nodes, cells=mesh.cells, cell_markers=mesh.cell_markers,
        node_markers=mesh.node_markers, boundaries=mesh.boundaries,
        boundary_markers=mesh.boundary_markers, boundary_cells=mesh.boundary_cells,
        sensors=data.sensorPositions(), abmn=data.abmn(), kfac=data["k"], k=k, w=w, rho=rho, rhoa=rhoa,
        primary=prim.reshape(len(k), data.sensorCount(), n)[0], subpot=sub[0], J=J,
        electrode_nodes=R.electrode_nodes())
    R.close()
    print(name, mesh, len(data), "k:", len(k), "J:", J.shape)


def main():
    xs = np.arange(7.0)
    m2 = create_para_mesh_2d(xs, para_dx=0.25, para_depth=3.0)
    case("ert2d_topo_sr_small", *_topo_2d(m2, xs), seed=31)
    e = np.array([(x, y) for x in (0.0, 4.0) for y in (0.0, 4.0)] + [(2.0, 0.0), (2.0, 4.0)])
    m3 = create_box_mesh_3d(e, h=1.0, para_margin=(1, 1), para_depth=3.0, outer=30.0, growth=2.0, depth_growth=1.5)
    m3n = Mesh(3, m3.nodes, m3.cells, m3.cell_markers, m3.node_markers, m3.boundaries, m3.boundary_markers,
               m3.boundary_cells, check=False)
    ab3 = np.array([[0, 1, 2, 3], [0, 2, 1, 3], [0, 4, 1, 5], [4, 5, 0, 3], [1, 3, 4, 2], [0, 3, 4, 5],
                    [2, 3, 0, 4], [5, 2, 1, 0]], np.int32)
    case("ert3d_topo_sr_small", *_topo_3d(m3n, e, ab3), seed=32)


if __name__ == "__main__":
    main()
