"""Generate the fixtures of the dipole current pattern from the reference's
own C++ (oracle/_ref/libgimli_ref.so, built by ``make -C oracle``) through
oracle/ref_driver.py:

    python tests/golden/make_dipole_golden.py [fixture names ...]

The reference (core/src/bert/dcfemmodelling.cpp) with
setDipoleCurrentPattern(true) solves one current pattern per distinct (a, b)
pair of the data (createCurrentPattern 1488-1513, +1 at a, -1 at b; b = -1:
no sink, the current leaves at infinity or, in a closed domain, at the
calibration nodes) and calculate(DataContainerERT &) (1558-1618) writes each
datum's voltage u = pot_m - pot_n of its pattern (unit current).  No
reference electrode takes part (searchElectrodes_ picks the last electrode
only without the dipole pattern, 1054).

The closed-domain singularity-removal fixture takes its primary potentials
per dipole pattern from the reference's total-potential operator at 1 Ohm m
on createP2 with the same dipole patterns (given with setPrimaryPotential:
the reference's own internal solve has no factorization in this build);
``primary`` holds the first wavenumber's rows at the mesh's nodes and
``patterns`` their (a, b) pairs in the reference's order (the sorted pattern
index (a + 1)(nSensors + 1) + b + 1, DataContainerERT::
electrodeToCurrentPattern, core/src/bert/bertDataContainer.cpp:149-153).

Fixtures (inputs, k/w, resistivity, voltages ``u``, number of patterns):

  ert3d_dipole_sr_small         3-D box with mixed boundaries
  ert3d_dipole_tp_small
  ert3d_dipole_closed_tp_small  closed 3-D box with a calibration node (-1000)
  ert3d_dipole_closed_sr_small  and a reference node (-999, unused)
  ert2d_dipole_sr_small         2.5-D line with mixed boundaries
  ert2d_dipole_tp_small
  ert2d_dipole_cem_small        the complete-electrode-model and bypass
  ert3d_dipole_cem_small        meshes of make_cem_golden.py (total potential,
  ert2d_dipole_bypass_small     their contact impedances and wavenumbers)

Run from the repository root.
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

from make_cem_golden import _resistivity  # noqa: E402
from oracle.ref_driver import RefModelling  # noqa: E402
from pygimli_gb300.data import DataContainerERT, createData  # noqa: E402
from pygimli_gb300.mesh import Mesh, create_box_mesh_3d, create_para_mesh_2d  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
only = set(sys.argv[1:])


def dipole_patterns(abmn, n_sensors):
    """(a, b) of the distinct current patterns in the reference's order."""
    ab = np.asarray(abmn, np.int64).reshape(-1, 4)[:, :2]
    idx = np.unique((ab[:, 0] + 1) * (n_sensors + 1) + ab[:, 1] + 1)
    return np.column_stack([idx // (n_sensors + 1) - 1, idx % (n_sensors + 1) - 1])


def case(name, mesh, data, seed, sr, numerical=False, contact_impedance=None, kw=None, rho=None):
    if only and name not in only:
        return
    ones = np.ones(data.size())
    R = RefModelling(mesh, data.sensorPositions(), data.abmn(), ones, sr=sr, contact_impedance=contact_impedance)
    if kw is not None:
        R.set_kw(*kw)
    k, w = R.kw()
    prim = np.zeros(0)
    if numerical:
        T = RefModelling(mesh, data.sensorPositions(), data.abmn(), ones, sr=False, p2=True)
        T.set_kw(k, w)
        T.calculate_dipole(np.ones(T.mesh_arrays()[2].shape[0]))
        sub = T.subpotentials()
        T.close()
        full = sub[:, :mesh.nodeCount()].copy()
        R.set_kw(k, w)
        R.set_primary(full)
        prim = full[:len(full) // len(k)]
    rho = _resistivity(mesh, seed) if rho is None else rho
    here = os.getcwd()
    with tempfile.TemporaryDirectory() as tmp:
        os.chdir(tmp)  # the reference's CEM path writes a debug matrix file into the working directory
        try:
            u, npat = R.calculate_dipole(rho)
        finally:
            os.chdir(here)
    pats = dipole_patterns(data.abmn(), data.sensorCount())
    assert len(pats) == npat
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"),
        dim=mesh.dim(), nodes=mesh.nodes, cells=mesh.cells, cell_markers=mesh.cell_markers,
        node_markers=mesh.node_markers, boundaries=mesh.boundaries, boundary_markers=mesh.boundary_markers,
        boundary_cells=mesh.boundary_cells, sensors=data.sensorPositions(), abmn=data.abmn(), k=k, w=w,
        rho=rho, u=u, n_patterns=npat, patterns=pats, primary=prim, sr=int(bool(sr)),
        contact_impedance=np.zeros(0) if contact_impedance is None else contact_impedance)
    R.close()
    print(name, mesh, len(data), "k:", len(k), "patterns:", npat)


def _remark(m, bm=None, nm=None):
    return Mesh(m.dim(), m.nodes, m.cells, m.cell_markers, m.node_markers if nm is None else nm, m.boundaries,
                m.boundary_markers if bm is None else bm, m.boundary_cells, check=False)


def _nearest(m, p):
    return int(np.argmin(np.linalg.norm(m.nodes - np.asarray(p, float), axis=1)))


def main():
    e = np.array([(x, y) for x in (0.0, 2.0, 4.0) for y in (0.0, 2.0)], float)
    m3 = create_box_mesh_3d(e, h=1.0, para_margin=(1, 1), para_depth=3.0, outer=12.0, growth=2.0,
                            depth_growth=1.5)
    # repeated, reversed and pole (b = -1) current pairs
    ab = np.array([[0, 1, 2, 3], [0, 2, 4, 5], [1, 3, 4, 5], [5, 0, 1, 2], [2, 5, 0, 1], [0, -1, 5, 3],
                   [3, 4, 1, 0], [4, 1, 3, 2], [0, 1, 4, 5], [1, 0, 2, 3], [2, 3, -1, 4]], np.int32)
    d3 = DataContainerERT(np.column_stack([e, np.zeros(len(e))]), ab)
    case("ert3d_dipole_sr_small", m3, d3, seed=61, sr=True)
    case("ert3d_dipole_tp_small", m3, d3, seed=62, sr=False)
    closed = _remark(m3, bm=np.full(len(m3.boundary_markers), -1, np.int32))
    nm = closed.node_markers.copy()
    ref = _nearest(closed, (2.0, 1.0, -3.0))
    cal = _nearest(closed, closed.nodes.min(axis=0))
    assert nm[ref] == 0 and nm[cal] == 0 and ref != cal
    nm[ref] = -999
    nm[cal] = -1000
    closed = _remark(closed, nm=nm)
    case("ert3d_dipole_closed_tp_small", closed, d3, seed=63, sr=False)
    case("ert3d_dipole_closed_sr_small", closed, d3, seed=64, sr=True, numerical=True)
    xs = np.arange(7.0)
    m2 = create_para_mesh_2d(xs, para_dx=0.25, para_depth=3.0)
    d2 = createData(xs, "dd")
    case("ert2d_dipole_sr_small", m2, d2, seed=65, sr=True)
    case("ert2d_dipole_tp_small", m2, d2, seed=66, sr=False)
    for src, name in (("ert2d_cem_small", "ert2d_dipole_cem_small"), ("ert3d_cem_small", "ert3d_dipole_cem_small"),
                      ("ert2d_bypass_small", "ert2d_dipole_bypass_small")):
        z = np.load(os.path.join(OUT, src + ".npz"))
        mz = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"], z["boundaries"],
                  z["boundary_markers"], z["boundary_cells"], check=False)
        zc = z["contact_impedance"]
        case(name, mz, DataContainerERT(z["sensors"], z["abmn"]), seed=0, sr=False,
             contact_impedance=zc if len(zc) else None, kw=(z["k"], z["w"]), rho=z["rho"])


if __name__ == "__main__":
    main()
