"""Singularity removal on a topographic surface (ERTModelling() on a mesh
whose surface is not flat).  The reference computes the primary potentials
numerically there: the total potential at 1 Ohm m on createP2 of the mesh,
taken at the mesh's nodes (DCSRMultiElectrodeModelling::checkPrimpotentials_,
core/src/bert/dcfemmodelling.cpp:2008-2068).  Fixtures from the reference's
own C++ (tests/golden/make_sr_topo_golden.py).

CPU: the oracle restatement (numerical primaries, then singularity removal
with them) against the fixtures.  GPU: the operator against the fixtures:
primary potentials <= 1e-9 of their maximum, potentials and apparent
resistivities <= 1e-6, Jacobian <= 1e-5 in the Frobenius norm, in every
solver form."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))

from oracle import ert_oracle as O  # noqa: E402
from pygimli_gb300.data import DataContainerERT  # noqa: E402
from pygimli_gb300.mesh import Mesh  # noqa: E402

CASES = ["ert2d_topo_sr_small", "ert3d_topo_sr_small"]
WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "pygimli_gb300", "weights")


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
    prim = O.numerical_primary(mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"])
    assert rel(prim[0], z["primary"]) <= 1e-9
    P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"], primary=prim)
    rhoa, u = P.response(z["rho"])
    assert float(np.max(np.abs(rhoa - z["rhoa"]) / z["rhoa"])) <= 1e-9
    assert rel(u[0], z["subpot"]) <= 1e-9
    J = P.jacobian(u, z["rho"])
    assert float(np.linalg.norm(J - z["J"]) / np.linalg.norm(z["J"])) <= 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "mixed", "mixed-fsai", "learned"])
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference(golden_dir, name, form):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pygimli_gb300 import ERTModelling
    z, mesh, data = load(golden_dir, name)
    kw = {"fp64": dict(precision="fp64"), "mixed": dict(precision="mixed"),
          "mixed-fsai": dict(precision="mixed", precond="fsai"),
          "learned": dict(precision="mixed", precond="learned",
                          weights=os.path.join(WEIGHTS, "line_2d.npz" if mesh.dim() == 2 else "box_3d.npz"))}[form]
    fop = ERTModelling(**kw)
    fop.setkValues(z["k"])
    fop.setWeights(z["w"])
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    rhoa = fop.response(z["rho"])
    e_prim = rel(fop.primaryPotentials()[0], z["primary"])
    e_pot = rel(fop.subPotentials()[0], z["subpot"])
    e_rhoa = float(np.max(np.abs(rhoa - z["rhoa"]) / z["rhoa"]))
    jdt = "float64" if form == "fp64" else "float32"
    J = fop.createJacobian(z["rho"], dtype=jdt).cpu().numpy().astype(np.float64)
    e_J = float(np.linalg.norm(J - z["J"]) / np.linalg.norm(z["J"]))
    print(f"{name} {form}: primary {e_prim:.2e} potentials {e_pot:.2e} rhoa {e_rhoa:.2e} J {e_J:.2e}")
    assert e_prim <= 1e-9 and e_pot <= 1e-6 and e_rhoa <= 1e-6 and e_J <= 1e-5
