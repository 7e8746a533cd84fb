"""Closed (Neumann-only) domains, reference and calibration nodes and
homogeneous Dirichlet boundaries, against fixtures from the reference's own
C++ (tests/golden/make_neumann_golden.py).

The reference (core/src/bert/dcfemmodelling.cpp): a mesh without mixed and
Dirichlet boundaries is a Neumann domain (711-773), treated as topography;
in 3-D the potential is fixed at calibration nodes (node marker -1000, else
node 0) and every current pattern returns through a reference electrode
(node marker -999, else the last electrode, 1011-1073, 1515-1523).  A
reference node gives (electrode, reference) patterns in any domain;
homogeneous Dirichlet boundaries (-3) clean their nodes' rows and columns.

CPU: the oracle restatement against the fixtures (matrix, sub-potentials,
apparent resistivities, Jacobian; with the reference at the last electrode
the reference's createJacobian stops, and the Jacobian is checked against
the reference's formula on its own sub-potentials and, for total
potentials, against central differences of the reference's response).
GPU: the operator against the same fixtures in every solver form: apparent
resistivities and potentials <= 1e-6, Jacobian <= 1e-5 (Frobenius), central
differences <= 1e-3."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))

import cem_oracle as CO  # noqa: E402
from oracle import ert_oracle as O  # noqa: E402
from pygimli_gb300.data import DataContainerERT  # noqa: E402
from pygimli_gb300.mesh import Mesh  # noqa: E402

CASES = ["ert3d_neumann_tp_small", "ert3d_neumann_sr_small", "ert3d_neumann_ref_tp_small",
         "ert3d_neumann_ref_sr_small", "ert3d_refnode_sr_small", "ert3d_refnode_tp_small",
         "ert3d_dirichlet_sr_small", "ert3d_dirichlet_tp_small", "ert2d_neumann_sr_small",
         "ert2d_neumann_tp_small"]
WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "pygimli_gb300", "weights")
TOL_FD = 1e-3


def load(golden_dir, name):
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"], z["boundaries"],
                z["boundary_markers"], z["boundary_cells"], check=False)
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", z["kfac"])
    return z, mesh, data


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def padded(z, rows, nE):
    """The reference keeps no pattern for a reference at the last electrode:
    its rows are those of electrodes 0..nE-2; here the last one is empty."""
    out = np.zeros((nE,) + rows.shape[1:])
    out[:len(rows)] = rows
    return out


def reciprocal_rows(z, mesh, data):
    """Data whose reciprocal configuration gives the same voltage (oracle,
    within 1e-6), with the sign of the voltage.  The response is
    sqrt(|r rr|) of the normal and the reciprocal voltages (dcfemmodelling.cpp:
    1133-1196); the Jacobian is that of k r alone, so only these rows of it
    are derivatives of the response: with the reference at the last
    electrode a datum that measures on that electrode has a reciprocal that
    injects there and differs."""
    P = oracle_problem(z, mesh, data)
    _, u = P.response(z["rho"])
    U = P.collect(u)
    r = O.Problem.data_u(P, U)
    rr = O.Problem.data_u(P, U, True)
    ok = np.abs(r - rr) <= 1e-6 * np.abs(r)
    return np.nonzero(ok)[0], np.sign(r * z["kfac"])


def fd_error(J, z, rows, sign):
    """Largest error of the Jacobian's columns fd_params on the given rows
    against the reference's central differences of the response, relative
    to the largest difference."""
    fd = z["fd_J"][rows]
    Jc = J[rows][:, z["fd_params"]] * sign[rows, None]
    return float(np.max(np.abs(Jc - fd)) / np.max(np.abs(fd)))


def reference_formula_J(z, mesh, data):
    """Where the reference's createJacobian stops (reference at the last
    electrode): its Jacobian formula (core/src/bert/bertJacobian.cpp:70-119,
    one wavenumber) on its own sub-potentials, the last electrode's pattern
    empty.  With singularity removal on a closed domain the normal and
    reciprocal voltages differ far beyond a derivative check, so this is the
    pin there; for total potentials the central differences of the
    response check it as well."""
    P = oracle_problem(z, mesh, data)
    u = padded(z, z["subpot"], data.sensorCount())[None]
    if not int(z["sr"]):
        u = np.concatenate([u, np.zeros(u.shape[:2] + (P.N - P.n,))], axis=2)
    return P.jacobian(u, z["rho"])


def oracle_problem(z, mesh, data):
    nE = data.sensorCount()
    if int(z["sr"]):
        prim = None
        if z["primary"].size:  # numerical primaries (all wavenumbers), pinned by the first one's
            prim = O.numerical_primary(mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"])
            assert rel(prim[0], padded(z, z["primary"], nE)) <= 1e-8
        return O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"], primary=prim)
    return CO.TotalPotentialProblem(mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"])


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(golden_dir, name):
    z, mesh, data = load(golden_dir, name)
    nE = data.sensorCount()
    P = oracle_problem(z, mesh, data)
    # the factored system matrix of the first wavenumber
    if int(z["sr"]):
        S = P.csr(P.assemble(z["rho"], 0))
    else:
        S = P.matrix(z["rho"], 0)
    R = O.sp.csr_matrix((z["S"], z["colidx"], z["rowptr"]), shape=S.shape)
    assert abs(S - R).max() <= 1e-12 * abs(R).max()
    rhoa, u = P.response(z["rho"])
    assert float(np.max(np.abs(rhoa - z["rhoa"]) / z["rhoa"])) <= 1e-9
    # a closed 2.5-D domain is nearly singular at the smallest wavenumber
    # (potentials ~1e5 there): two direct solves agree to a few 1e-9
    tol_u = 1e-8 if name.startswith("ert2d_neumann") else 1e-9
    assert rel(u[0][:, :mesh.nodeCount()], padded(z, z["subpot"], nE)) <= tol_u
    J = P.jacobian(u, z["rho"])
    if "J" in z:
        assert float(np.linalg.norm(J - z["J"]) / np.linalg.norm(z["J"])) <= 1e-9
    else:
        Jr = reference_formula_J(z, mesh, data)
        assert float(np.linalg.norm(J - Jr) / np.linalg.norm(Jr)) <= 1e-9
        if not int(z["sr"]):
            rows, sign = reciprocal_rows(z, mesh, data)
            assert len(rows) >= len(J) // 2
            assert fd_error(J, z, rows, sign) <= TOL_FD


def test_setup_rules(golden_dir):
    """Calibration and reference choice of the reference's searchElectrodes_."""
    _, closed, data = load(golden_dir, "ert3d_neumann_tp_small")
    bc = O.BoundarySetup(closed, data.sensorCount())
    assert bc.neumann and bc.topography and list(bc.calib) == [0] and bc.ref_elec == data.sensorCount() - 1
    _, m, _ = load(golden_dir, "ert3d_neumann_ref_tp_small")
    bc = O.BoundarySetup(m, data.sensorCount())
    assert bc.ref_elec == -1 and bc.ref_node == int(np.nonzero(m.node_markers == -999)[0][0])
    assert list(bc.calib) == list(np.nonzero(m.node_markers == -1000)[0])
    _, m, _ = load(golden_dir, "ert3d_refnode_tp_small")
    bc = O.BoundarySetup(m, data.sensorCount())
    assert not bc.neumann and len(bc.calib) == 0 and bc.ref_node >= 0 and len(bc.dirichlet) == 0
    _, m, _ = load(golden_dir, "ert3d_dirichlet_tp_small")
    bc = O.BoundarySetup(m, data.sensorCount())
    assert not bc.neumann and not bc.topography and len(bc.dirichlet) > 0 and len(bc.calib) == 0
    _, m, d2 = load(golden_dir, "ert2d_neumann_tp_small")
    bc = O.BoundarySetup(m, d2.sensorCount())
    assert bc.neumann and bc.topography and len(bc.calib) == 0 and bc.ref_elec == -1


def test_numerical_primary_matches_reference(golden_dir):
    """The oracle's numerical primaries (total potential at 1 Ohm m on
    createP2) of a closed box with reference and calibration nodes."""
    z, mesh, data = load(golden_dir, "ert3d_neumann_ref_sr_small")
    prim = O.numerical_primary(mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"])
    assert rel(prim[0], z["primary"]) <= 1e-9


def test_host_setup_matches_oracle(golden_dir):
    """The operator's host-side boundary setup (pygimli_gb300.ert) picks the
    oracle's calibration nodes, reference and topography flag."""
    from pygimli_gb300.ert import boundary_setup
    for name in CASES:
        z, mesh, data = load(golden_dir, name)
        ours = boundary_setup(mesh, data.sensorCount())
        bc = O.BoundarySetup(mesh, data.sensorCount())
        assert ours.neumann == bc.neumann and ours.topography == bc.topography, name
        assert list(ours.calib) == list(bc.calib) and list(ours.dirichlet) == list(bc.dirichlet), name
        assert ours.ref_node == bc.ref_node and ours.ref_elec == bc.ref_elec, name


FORMS = {"fp64": dict(precision="fp64"), "mixed": dict(precision="mixed"),
         "mixed-fsai": dict(precision="mixed", precond="fsai")}


@pytest.mark.gpu
@pytest.mark.parametrize("form", list(FORMS) + ["learned"])
@pytest.mark.parametrize("name", CASES)
def test_gpu_matches_reference(golden_dir, name, form):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pygimli_gb300 import ERTModelling
    z, mesh, data = load(golden_dir, name)
    nE = data.sensorCount()
    sr = bool(int(z["sr"]))
    if form == "learned":
        kw = dict(precision="mixed", precond="learned",
                  weights=os.path.join(WEIGHTS, "line_2d.npz" if mesh.dim() == 2 else "box_3d.npz"))
    else:
        kw = dict(FORMS[form])
    fop = ERTModelling(sr=sr, **kw)
    fop.setkValues(z["k"])
    fop.setWeights(z["w"])
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    rhoa = fop.response(z["rho"])
    e_pot = rel(fop.subPotentials()[0][:, :mesh.nodeCount()], padded(z, z["subpot"], nE))
    e_rhoa = float(np.max(np.abs(rhoa - z["rhoa"]) / z["rhoa"]))
    jdt = "float64" if form == "fp64" else "float32"
    J = fop.createJacobian(z["rho"], dtype=jdt).cpu().numpy().astype(np.float64)
    msg = f"{name} {form}: potentials {e_pot:.2e} rhoa {e_rhoa:.2e}"
    Jr = z["J"] if "J" in z else reference_formula_J(z, mesh, data)
    e_J = float(np.linalg.norm(J - Jr) / np.linalg.norm(Jr))
    msg += f" J {e_J:.2e}"
    if "J" not in z and not sr:
        rows, sign = reciprocal_rows(z, mesh, data)
        e_fd = fd_error(J, z, rows, sign)
        msg += f" (central differences {e_fd:.2e})"
        assert e_fd <= TOL_FD
    print(msg)
    assert e_J <= 1e-5
    assert e_pot <= 1e-6 and e_rhoa <= 1e-6


@pytest.mark.gpu
def test_gpu_error_paths(golden_dir):
    """Through the C ABI: a closed 3-D domain without calibration node is
    refused (STATE); complex resistivity refuses a reference electrode."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from pygimli_gb300 import ERTModelling
    from pygimli_gb300._native import BAD_INPUT, STATE, ErtgbError
    z, mesh, data = load(golden_dir, "ert3d_neumann_tp_small")
    fop = ERTModelling(sr=False)
    fop.setkValues(z["k"])
    fop.setWeights(z["w"])
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    assert fop._lib.ertgb_set_reference(fop._ctx, -1, -1, 0, None) == 0
    rho = torch.tensor(z["rho"], device="cuda")
    out = torch.empty(data.size(), dtype=torch.float64, device="cuda")
    import ctypes
    rc = fop._lib.ertgb_response(fop._ctx, ctypes.c_void_p(rho.data_ptr()), ctypes.c_void_p(out.data_ptr()), None)
    assert rc == STATE and b"calibration" in fop._lib.ertgb_last_error(fop._ctx)
    fop.setData(data)  # the operator's own setup again
    r = fop.response(z["rho"])
    assert float(np.max(np.abs(r - z["rhoa"]) / z["rhoa"])) <= 1e-6
    fop.setComplex(True)
    with pytest.raises(ErtgbError) as e:
        fop.response(np.concatenate([z["rho"], np.full(len(z["rho"]), -1e-3)]))
    assert e.value.code == BAD_INPUT
