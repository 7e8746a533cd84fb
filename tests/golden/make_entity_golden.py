"""Generate the fixtures of electrodes that are not mesh nodes, by running
the reference's own C++ (oracle/_ref/libgimli_ref.so, built by
``make -C oracle``) through oracle/ref_driver.py:

    python tests/golden/make_entity_golden.py

A sensor that matches no electrode node (and no CEM or bypass electrode)
becomes an ElectrodeShapeEntity of the cell that holds it
(DCMultiElectrodeModelling::searchElectrodes_, core/src/bert/
dcfemmodelling.cpp:924-937; core/src/bert/electrode.cpp:252-290): the source
enters with the cell's shape functions at the sensor, the electrode
potential is the interpolation there, the source resistivity is the cell's.
The sensors lie on the surface between electrode nodes, inside one surface
face each, so that exactly one cell holds each of them.

  ert2d_entity_small    2.5-D, singularity removal, 7 sensors at x = i + 0.125
  ert3d_entity_small    3-D, singularity removal, 6 sensors off the nodes
  ert2d_entity_tp_small 2.5-D, total potential, the sensors of ert2d_entity_small

Run from the repository root.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.ref_driver import RefModelling  # noqa: E402
from pygimli_gb300.data import DataContainerERT, createData, geometricFactors  # noqa: E402
from pygimli_gb300.mesh import create_box_mesh_3d, create_para_mesh_2d  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def case(name, mesh, data, seed, sr=True):
    R = RefModelling(mesh, data.sensorPositions(), data.abmn(), data["k"], sr=sr)
    k, w = R.kw()
    rng = np.random.default_rng(seed)
    rho = np.exp(rng.uniform(np.log(50.0), np.log(200.0), mesh.cellCount()))
    rhoa = R.response(rho)
    sub = R.subpotentials().reshape(len(k), data.sensorCount(), -1)
    J = R.jacobian(rho)
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"),
        dim=mesh.dim(), nodes=mesh.nodes, cells=mesh.cells, cell_markers=mesh.cell_markers,
        node_markers=mesh.node_markers, boundaries=mesh.boundaries,
        boundary_markers=mesh.boundary_markers, boundary_cells=mesh.boundary_cells,
        sensors=data.sensorPositions(), abmn=data.abmn(), kfac=data["k"], k=k, w=w, rho=rho, rhoa=rhoa,
        subpot_first=sub[0], subpot_last=sub[-1], J=J, sr=int(sr))
    R.close()
    print(name, mesh, len(data), "k:", len(k), "J:", J.shape)


def main():
    xs = np.arange(7.0)
    m2 = create_para_mesh_2d(xs, para_dx=0.25, para_depth=3.0)
    d2 = DataContainerERT(np.column_stack([xs + 0.125, np.zeros(7), np.zeros(7)]), createData(xs, "dd").abmn())
    d2["k"] = geometricFactors(d2, 2)
    case("ert2d_entity_small", m2, d2, seed=41)
    case("ert2d_entity_tp_small", m2, d2, seed=43, sr=False)
    e = np.array([(x, y) for x in (0.0, 4.0) for y in (0.0, 4.0)] + [(2.0, 0.0), (2.0, 4.0)])
    m3 = create_box_mesh_3d(e, h=1.0, para_margin=(1, 1), para_depth=3.0, outer=30.0, growth=2.0, depth_growth=1.5)
    s3 = np.column_stack([e[:, 0] + 0.3, e[:, 1] + 0.15, np.zeros(len(e))])
    ab3 = np.array([[0, 1, 2, 3], [0, 2, 1, 3], [0, 4, 1, 5], [4, 5, 0, 3], [1, 3, 4, 2], [0, 3, 4, 5],
                    [2, 3, 0, 4], [5, 2, 1, 0]], np.int32)
    d3 = DataContainerERT(s3, ab3)
    d3["k"] = geometricFactors(d3, 3)
    case("ert3d_entity_small", m3, d3, seed=42)


if __name__ == "__main__":
    main()
