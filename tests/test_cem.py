"""The total-potential operator (pyGIMLi ERTModelling(sr=False), the
reference's DCMultiElectrodeModelling) with node, complete-electrode-model
(CEM) and bypass electrodes.

CPU: the oracle restatement (oracle/cem_oracle.py) against the fixtures the
reference's own C++ produced (tests/golden/make_cem_golden.py), and the
product's host-side electrode search and matrix extension
(pygimli_gb300/cem.py) against the reference's assembled matrix.
GPU (marked): response and Jacobian through ERTModelling against the same
fixtures.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest
import scipy.sparse as sp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import cem_oracle as CO  # noqa: E402
from pygimli_gb300 import cem  # noqa: E402
from pygimli_gb300.data import DataContainerERT  # noqa: E402
from pygimli_gb300.mesh import Mesh  # noqa: E402

CASES = ["ert2d_tp_small", "ert2d_cem_small", "ert3d_cem_small", "ert2d_bypass_small", "ert2d_topo_tp_small",
         "ert3d_topo_tp_small", "ert2d_cem_p2_small", "ert3d_cem_p2_small"]
TOPO = ["ert2d_topo_tp_small", "ert3d_topo_tp_small"]


def load(golden_dir, name):
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"], z["boundaries"],
                z["boundary_markers"], z["boundary_cells"], check=False)
    if "p2" in z.files and int(z["p2"]) == 1:
        mesh = mesh.createP2()   # the reference's numbering (tests/test_refine.py)
    zc = z["contact_impedance"]
    return z, mesh, (zc if len(zc) else None)


def ref_matrix(z):
    N = len(z["rowptr"]) - 1
    return sp.csr_matrix((z["S"], z["colidx"], z["rowptr"]), shape=(N, N))


# ------------------------------------------------------------------ CPU --
@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(golden_dir, name):
    """The oracle's total-potential operator against the reference: the
    assembled matrix (first wavenumber) to rounding, sub-potentials,
    apparent resistivities and the Jacobian.  The bypass case carries 1e-6
    Ohm resistors next to ~0.01 S element entries: the direct solves of the
    reference and of scipy then differ in the 9th digit."""
    z, mesh, zc = load(golden_dir, name)
    P = CO.TotalPotentialProblem(mesh, z["sensors"], z["abmn"], z["kfac"], z["k"], z["w"], contact_impedance=zc)
    if len(z["S"]):
        R = ref_matrix(z)
        A = P.matrix(z["rho"], 0)
        assert A.shape == R.shape and A.nnz == R.nnz
        assert abs(A - R).max() <= 1e-15 * abs(R).max()
    rhoa, u = P.response(z["rho"])
    J = P.jacobian(u, z["rho"])
    tol = 1e-7 if "bypass" in name else 1e-12
    assert np.max(np.abs(rhoa - z["rhoa"]) / np.abs(z["rhoa"])) <= tol
    assert np.max(np.abs(J - z["J"])) <= tol * np.max(np.abs(z["J"]))
    assert np.max(np.abs(u[0, :, :P.n] - z["subpot_first"])) <= 100 * tol * np.max(np.abs(z["subpot_first"]))


def test_oracle_cem_collects_last_wavenumber(golden_dir):
    """With CEM in 2.5-D the reference's electrode potentials are those of
    its last wavenumber, unweighted: the oracle's k-summed potentials do not
    reproduce its apparent resistivities, the last-wavenumber ones do."""
    z, mesh, zc = load(golden_dir, "ert2d_cem_small")
    P = CO.TotalPotentialProblem(mesh, z["sensors"], z["abmn"], z["kfac"], z["k"], z["w"], contact_impedance=zc)
    assert P.cem and len(P.k) > 1
    u = P.solve(z["rho"])
    U_sum = np.einsum("k,ken->en", P.w, u)[:, P.src_row]
    r = CO.Problem.data_u(P, U_sum) * P.kfac
    assert np.max(np.abs(np.abs(r) - z["rhoa"]) / z["rhoa"]) > 10.0


@pytest.mark.parametrize("name", CASES)
def test_host_extension_matches_reference(golden_dir, name):
    """pygimli_gb300.cem (closed-form entity integrals) builds the entries
    the reference adds to its matrix: reference matrix minus the element and
    boundary terms equals the summed extension entries."""
    z, mesh, zc = load(golden_dir, name)
    setup = cem.electrode_setup(mesh, z["sensors"], contact_impedance=zc)
    P = CO.TotalPotentialProblem(mesh, z["sensors"], z["abmn"], z["kfac"], z["k"], z["w"], contact_impedance=zc)
    # without the reference's matrix in the fixture: the oracle's, which
    # reproduces the reference's apparent resistivities and Jacobian
    R = ref_matrix(z) if len(z["S"]) else P.matrix(z["rho"], 0)
    P.ext, P.ext_diag = {}, {}
    fem = P.matrix(z["rho"], 0)
    N = R.shape[0]
    assert mesh.nodeCount() + setup.n_ext == N
    X = sp.csr_matrix((setup.vals, (setup.rows, setup.cols)), shape=(N, N))
    D = (R - fem) - X
    assert abs(D).max() <= 1e-12 * max(abs(R).max(), 1.0)
    # electrode rows and positions as the oracle's search finds them
    np.testing.assert_array_equal(setup.src_row, P.src_row)
    np.testing.assert_allclose(setup.src_center, P.src_center, rtol=0, atol=1e-13)
    assert setup.cem == P.cem
    assert [e.kind for e in setup.electrodes] == [e.kind for e in P.electrodes]


@pytest.mark.parametrize("name", TOPO)
def test_oracle_electrode_potentials_topography(golden_dir, name):
    """On a surface with topography (total potential only) the oracle's
    k-summed electrode potential matrix equals the reference's for the model
    and for 1 Ohm m, and the product's DataMap voltages equal the oracle's."""
    from pygimli_gb300.ert import datamap_voltages
    z, mesh, _ = load(golden_dir, name)
    P = CO.TotalPotentialProblem(mesh, z["sensors"], z["abmn"], z["kfac"], z["k"], z["w"])
    U = P.collect(P.solve(z["rho"]))
    U1 = P.collect(P.solve(np.ones(mesh.cellCount())))
    assert np.abs(U - z["U"]).max() <= 1e-13 * np.abs(z["U"]).max()
    assert np.abs(U1 - z["U1"]).max() <= 1e-13 * np.abs(z["U1"]).max()
    np.testing.assert_array_equal(datamap_voltages(U, z["abmn"]), CO.Problem.data_u(P, U))


def test_datamap_voltages_with_poles():
    """DataMap voltages with electrodes at infinity (index -1 in a, b or n)
    equal the oracle's restatement of DataMap::data."""
    from pygimli_gb300.ert import datamap_voltages
    rng = np.random.default_rng(5)
    U = rng.normal(size=(6, 6))
    ab = np.array([[0, 1, 2, 3], [0, -1, 2, 3], [-1, 1, 4, 5], [2, 3, 4, -1], [5, -1, 0, -1], [1, 4, 3, 2]])

    class _P:
        abmn = ab

    np.testing.assert_array_equal(datamap_voltages(U, ab), CO.Problem.data_u(_P, U))
    assert datamap_voltages(U, ab)[4] == U[5, 0]


def test_entity_integrals_closed_form():
    """Closed-form integrals of the product against the oracle's quadrature
    for every entity type (linear and quadratic)."""
    rng = np.random.default_rng(3)
    for nvert, dim_e, nc in ((2, 1, 2), (3, 1, 2), (3, 2, 3), (6, 2, 3), (4, 3, 4), (10, 3, 4)):
        corners = rng.normal(size=(nc, 3))
        u, u2 = cem.entity_integrals(nvert, corners)
        uo, u2o = CO.entity_integrals(dim_e, corners, nvert)
        np.testing.assert_allclose(u, uo, rtol=1e-13, atol=1e-15)
        np.testing.assert_allclose(u2, u2o, rtol=1e-13, atol=1e-15)


def test_mark_cem_electrodes_and_search():
    """mark_cem_electrodes sets -10000 - i on the surface boundaries under
    each electrode and -9999 for a passive body; the search matches sensors
    to them and gives one extension row per electrode and passive body."""
    from pygimli_gb300.mesh import create_para_mesh_2d
    xs = np.arange(5.0)
    m = create_para_mesh_2d(xs, para_dx=0.25, para_depth=2.0)
    mc = cem.mark_cem_electrodes(m, np.column_stack([xs, np.zeros(5)]), 0.25, passive=[((2.5, 0.0), 0.25)])
    bm = mc.boundary_markers
    for i in range(5):
        assert np.count_nonzero(bm == cem.MARKER_BOUND_ELECTRODE - i) == 2
    assert np.count_nonzero(bm == cem.MARKER_BOUND_ELECTRODE + 1) == 2
    assert not np.any(mc.node_markers == cem.MARKER_NODE_ELECTRODE)
    s = cem.electrode_setup(mc, np.column_stack([xs, np.zeros(5), np.zeros(5)]))
    assert s.cem and s.n_ext == 6 and len(s.passive) == 1
    np.testing.assert_array_equal(s.src_row, mc.nodeCount() + np.arange(5))
    assert np.all(s.enode == -1)
    with pytest.raises(ValueError):
        cem.electrode_setup(mc, np.column_stack([xs, np.zeros(5), np.zeros(5)]), contact_impedance=np.ones(3))


def test_has_cem_markers(golden_dir):
    """CEM boundaries and bypass nodes are detected (ERTModelling(sr=True)
    refuses such meshes, tested on the GPU); plain meshes carry none."""
    for name, expect in (("ert3d_cem_small", True), ("ert2d_bypass_small", True), ("ert2d_tp_small", False)):
        _, mesh, _ = load(golden_dir, name)
        assert cem.has_cem_markers(mesh) == expect


# ------------------------------------------------------------------ GPU --
@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    from pygimli_gb300 import build
    build.build()
    return t


def _fop(z, mesh, zc, **kw):
    from pygimli_gb300 import ERTModelling
    fop = ERTModelling(sr=False, **kw)
    if zc is not None:
        fop.setContactImpedances(zc)
    fop.setkValues(z["k"])
    fop.setWeights(z["w"])
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", z["kfac"])
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    return fop


GPU_CASES = [("ert2d_tp_small", "fp64"), ("ert2d_tp_small", "mixed"), ("ert2d_tp_small", "mixed-fsai"),
             ("ert2d_cem_small", "fp64"), ("ert2d_cem_small", "mixed-fsai"),
             ("ert3d_cem_small", "fp64"), ("ert3d_cem_small", "mixed"), ("ert3d_cem_small", "mixed-fsai"),
             ("ert2d_bypass_small", "fp64"), ("ert2d_topo_tp_small", "fp64"), ("ert2d_topo_tp_small", "mixed-fsai"),
             ("ert3d_topo_tp_small", "fp64"), ("ert3d_topo_tp_small", "mixed-fsai"), ("ert3d_cem_p2_small", "fp64")]
FORMS = {"fp64": dict(precision="fp64"), "mixed": dict(precision="mixed"),
         "mixed-fsai": dict(precision="mixed", precond="fsai")}


@pytest.mark.gpu
@pytest.mark.parametrize("name,form", GPU_CASES)
def test_total_potential_golden(torch, golden_dir, name, form):
    """ERTModelling(sr=False) on the GPU against the reference: the
    assembled matrix with its CEM / bypass extension (1e-12), apparent
    resistivities and the Jacobian.  The PCG runs to rtol 1e-10 where the
    reference factors: rhoa within 1e-8, J within 1e-6 (relative norm); the
    bypass case's 1e-6 Ohm resistors raise the condition number by ~1e8,
    so there rhoa 2e-6 and J 1e-5.  (The 2.5-D P2 CEM fixture has voltages
    of one rounding step, 8e-13 from a rounding boundary: it is checked by
    the oracle only.)  The 2.5-D CEM response is the last
    wavenumber's unweighted electrode potential (the reference's collect):
    its far-electrode values are ~1e-8 while the response rounds to 1e-10,
    so the FP64 Jacobi solve runs to rtol 1e-12 there (at 1e-10 the error
    of ~5e-11 moves one voltage by half a rounding step; the same Jacobi PCG
    on the CPU reproduces both)."""
    z, mesh, zc = load(golden_dir, name)
    kw = dict(FORMS[form])
    if name == "ert2d_cem_small" and form == "fp64":
        kw["rtol"] = 1e-12
    fop = _fop(z, mesh, zc, **kw)
    rhoa = fop.response(z["rho"])
    if len(z["S"]):
        R = ref_matrix(z)
        rp, ci = fop.pattern()
        assert len(rp) - 1 == R.shape[0]
        S = sp.csr_matrix((fop.matrix(0), ci, rp), shape=R.shape)
        assert abs(S - R).max() <= 1e-12 * abs(R).max()
    J = fop.createJacobian(z["rho"]).cpu().numpy()
    e_r = float(np.max(np.abs(rhoa - z["rhoa"]) / np.abs(z["rhoa"])))
    e_j = float(np.linalg.norm(J - z["J"]) / np.linalg.norm(z["J"]))
    st = fop.stats()
    print(f"{name} {form}: rhoa {e_r:.2e} J {e_j:.2e} iterations {st['iterations']} "
          f"FP64-finished columns {st['stalled_columns']}")
    tol_r, tol_j = (2e-6, 1e-5) if "bypass" in name else (1e-8, 1e-6)
    assert e_r <= tol_r and e_j <= tol_j


@pytest.mark.gpu
def test_total_potential_guards(torch, golden_dir):
    """Refusals of the formulation: the SR operator on a CEM mesh, the
    learned preconditioner and complex resistivity with a matrix extension,
    data without geometric factors on a CEM mesh (the reference's response
    refuses them, dcfemmodelling.cpp:1088-1097); calcGeometricFactor there
    gives numerical factors: unit resistivity then has apparent resistivity 1."""
    from pygimli_gb300 import ERTModelling
    z, mesh, zc = load(golden_dir, "ert3d_cem_small")
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", z["kfac"])
    sr = ERTModelling()
    sr.setData(data)
    with pytest.raises(ValueError):
        sr.setMesh(mesh, ignoreRegionManager=True)
    fop = _fop(z, mesh, zc, precision="mixed", precond="learned",
               weights=os.path.join(ROOT, "pygimli_gb300", "weights", "box_3d.npz"))
    with pytest.raises(RuntimeError):
        fop.response(z["rho"])
    fop = _fop(z, mesh, zc)
    bare = DataContainerERT(z["sensors"], z["abmn"])
    with pytest.raises(ValueError, match="no K-factors"):
        fop.setData(bare)
    fop = _fop(z, mesh, zc)
    k_num = fop.calcGeometricFactor()
    unit = DataContainerERT(z["sensors"], z["abmn"])
    unit.set("k", k_num)
    fop.setData(unit)
    rhoa = fop.response(np.ones(mesh.cellCount()))
    assert np.max(np.abs(rhoa - 1.0)) <= 1e-6
    fop.setComplex(True)
    with pytest.raises(RuntimeError):
        fop.response(np.concatenate([z["rho"], -0.01 * z["rho"]]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", TOPO)
def test_simulate_calc_only_and_numerical_factors(torch, golden_dir, name):
    """simulate(sr=False, calcOnly=True) returns the reference's DataMap
    voltages (no rounding, no reciprocity) on a topographic surface;
    createGeometricFactors(numerical=True) is 1 / those voltages at 1 Ohm m;
    returnFields the k-summed potentials per source."""
    from pygimli_gb300.ert import createGeometricFactors, datamap_voltages, simulate
    z, mesh, _ = load(golden_dir, name)
    scheme = DataContainerERT(z["sensors"], z["abmn"])
    d = simulate(mesh, scheme, z["rho"], sr=False, calcOnly=True, current=2.0)
    u_ref = datamap_voltages(z["U"], z["abmn"])
    assert np.max(np.abs(d["r"] - u_ref) / np.abs(u_ref)) <= 1e-8
    np.testing.assert_allclose(d["u"], 2.0 * d["r"], rtol=1e-15)
    assert not scheme.allNonZero("k")
    k_num = createGeometricFactors(scheme, numerical=True, mesh=mesh, h2=False, p2=False)
    k_ref = 1.0 / datamap_voltages(z["U1"], z["abmn"])
    assert np.max(np.abs(k_num - k_ref) / np.abs(k_ref)) <= 1e-8
    sol = simulate(mesh, scheme, z["rho"], sr=False, calcOnly=True, returnFields=True)
    assert sol.shape == (scheme.sensorCount(), mesh.nodeCount())


@pytest.mark.gpu
@pytest.mark.parametrize("name", TOPO)
def test_numerical_factors_on_topography(torch, golden_dir, name):
    """On a topographic surface the operator refuses data without geometric
    factors (the reference computes them analytically only for a flat
    surface) and calcGeometricFactor gives the numerical ones: 1 / (u + 1e-12)
    with u the voltages at unit resistivity, pinned to the reference's own
    unit-resistivity electrode potentials (core/src/bert/dcfemmodelling.cpp:
    1527-1557)."""
    from pygimli_gb300 import ERTModelling
    from pygimli_gb300.ert import datamap_voltages
    z, mesh, _ = load(golden_dir, name)
    fop = ERTModelling(sr=False)
    fop.setkValues(z["k"])
    fop.setWeights(z["w"])
    with pytest.raises(ValueError, match="no K-factors"):
        fop.setData(DataContainerERT(z["sensors"], z["abmn"]))
        fop.setMesh(mesh, ignoreRegionManager=True)
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", np.ones(data.size()))
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    k_num = fop.calcGeometricFactor(DataContainerERT(z["sensors"], z["abmn"]))
    k_ref = 1.0 / (datamap_voltages(z["U1"], z["abmn"]) + 1e-12)
    assert np.max(np.abs(k_num - k_ref) / np.abs(k_ref)) <= 1e-8
