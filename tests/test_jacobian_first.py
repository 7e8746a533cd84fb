"""A Jacobian requested before any response (createJacobian on a fresh
operator): the reference then computes the sub-potentials itself
(prepareJacobianT_, core/src/bert/dcfemmodelling.cpp:1262-1301) --
analytically for a homogeneous model (scaled by its value), by a response to
the model otherwise.  Fixtures from the reference's own C++
(tests/golden/make_jacobian_first_golden.py).  CPU: the oracle restatement;
GPU: the operator (FP64 J), Frobenius error <= 1e-5 (observed ~1e-12 for the
analytic branch)."""
import os

import numpy as np
import pytest

from oracle import ert_oracle as O
from pygimli_gb300.data import DataContainerERT
from pygimli_gb300.mesh import Mesh


def load(golden_dir, name):
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"], z["boundaries"],
                z["boundary_markers"], z["boundary_cells"])
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", z["kfac"])
    return z, mesh, data


def frob(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("tag,name", [("2d", "ert2d_small"), ("3d", "ert3d_small")])
def test_oracle_analytic_branch(golden_dir, tag, name):
    f = np.load(os.path.join(golden_dir, "jacobian_first_small.npz"))
    z, mesh, data = load(golden_dir, name)
    P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"])
    rho = float(f["rho_hom"])
    J = P.jacobian(P.up * rho, np.full(mesh.cellCount(), rho))
    assert frob(J, f["J_hom_" + tag]) <= 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("tag,name", [("2d", "ert2d_small"), ("3d", "ert3d_small")])
def test_gpu_jacobian_before_response(golden_dir, tag, name):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pygimli_gb300 import ERTModelling
    f = np.load(os.path.join(golden_dir, "jacobian_first_small.npz"))
    z, mesh, data = load(golden_dir, name)
    errs = {}
    for kind, model in (("hom", np.full(mesh.cellCount(), float(f["rho_hom"]))), ("het", z["rho"])):
        fop = ERTModelling()
        fop.setkValues(z["k"])
        fop.setWeights(z["w"])
        fop.setData(data)
        fop.setMesh(mesh, ignoreRegionManager=True)
        J = fop.createJacobian(model).cpu().numpy()
        errs[kind] = frob(J, f[f"J_{kind}_{tag}"])
    print(f"{name}: Jacobian before any response, homogeneous {errs['hom']:.2e}, heterogeneous {errs['het']:.2e}")
    assert errs["hom"] <= 1e-5 and errs["het"] <= 1e-5
