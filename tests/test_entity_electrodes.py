"""Electrodes that are not mesh nodes (the reference's ElectrodeShapeEntity,
core/src/bert/electrode.cpp:252-290, chosen by searchElectrodes_,
core/src/bert/dcfemmodelling.cpp:924-937): the source enters with the shape
functions of the cell that holds the sensor, the electrode potential is the
interpolation there, the source resistivity is that cell's.  Fixtures from
the reference's own C++ (tests/golden/make_entity_golden.py).

CPU: the oracle restatement against the fixtures.  GPU: the operator against
the fixtures (potentials and apparent resistivities <= 1e-6, Jacobian <= 1e-5
in the Frobenius norm) for singularity removal and the total potential."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))

import cem_oracle as CO  # noqa: E402
from oracle import ert_oracle as O  # noqa: E402
from pygimli_gb300.data import DataContainerERT  # noqa: E402
from pygimli_gb300.mesh import Mesh  # noqa: E402

CASES = ["ert2d_entity_small", "ert3d_entity_small", "ert2d_entity_tp_small"]


def load(golden_dir, name):
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"], z["boundaries"],
                z["boundary_markers"], z["boundary_cells"], check=False)
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", z["kfac"])
    return z, mesh, data


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(golden_dir, name):
    z, mesh, data = load(golden_dir, name)
    if int(z["sr"]):
        P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"])
        assert np.all(P.enodes == -1)  # every sensor is off the electrode nodes
    else:
        P = CO.TotalPotentialProblem(mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"])
        assert all(e.kind == "entity" for e in P.electrodes)
    rhoa, u = P.response(z["rho"])
    assert float(np.max(np.abs(rhoa - z["rhoa"]) / z["rhoa"])) <= 1e-9
    assert rel(u[0], z["subpot_first"]) <= 1e-9 and rel(u[-1], z["subpot_last"]) <= 1e-9
    J = P.jacobian(u, z["rho"])
    assert float(np.linalg.norm(J - z["J"]) / np.linalg.norm(z["J"])) <= 1e-9


def test_host_search_finds_cells(golden_dir):
    """The host electrode search (singularity removal and total potential)
    falls back to the cell that holds the sensor, as the reference's."""
    from pygimli_gb300.cem import electrode_setup
    from pygimli_gb300.ert import search_electrodes
    for name in CASES:
        z, mesh, data = load(golden_dir, name)
        es = search_electrodes(mesh, data.sensorPositions())
        assert np.all(es.nodes == -1) and np.all(es.cells >= 0)
        P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"])
        assert np.array_equal(es.cells, [int(c[0]) for c in P.ecells])
        setup = electrode_setup(mesh, data.sensorPositions())
        assert setup.search is not None and np.array_equal(setup.search.cells, es.cells)


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "mixed-fsai"])
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference(golden_dir, name, form):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pygimli_gb300 import ERTModelling
    z, mesh, data = load(golden_dir, name)
    kw = dict(precision="fp64") if form == "fp64" else dict(precision="mixed", precond="fsai")
    fop = ERTModelling(sr=bool(int(z["sr"])), **kw)
    fop.setkValues(z["k"])
    fop.setWeights(z["w"])
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    rhoa = fop.response(z["rho"])
    u = fop.subPotentials()
    e_pot = max(rel(u[0], z["subpot_first"]), rel(u[-1], z["subpot_last"]))
    e_rhoa = float(np.max(np.abs(rhoa - z["rhoa"]) / z["rhoa"]))
    jdt = "float64" if form == "fp64" else "float32"
    J = fop.createJacobian(z["rho"], dtype=jdt).cpu().numpy().astype(np.float64)
    e_J = float(np.linalg.norm(J - z["J"]) / np.linalg.norm(z["J"]))
    print(f"{name} {form}: potentials {e_pot:.2e} rhoa {e_rhoa:.2e} J {e_J:.2e}")
    assert e_pot <= 1e-6 and e_rhoa <= 1e-6 and e_J <= 1e-5
