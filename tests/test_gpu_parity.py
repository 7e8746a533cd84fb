"""GPU parity of the CUDA path (libertgb.so through ERTModelling and the C ABI)
against the reference's own outputs (tests/golden/) and the FP64 oracle.

Tolerances (relative): CSR indices bit-exact; matrix values <= 1e-12;
primary potentials <= 1e-12; potentials and apparent resistivities <= 1e-6;
Jacobian <= 1e-5 in the Frobenius norm.  Full-size workloads are checked
through size-independent properties (linearity in the resistivity scale,
the half-space value, Jacobian rows recomputed from the GPU potentials)."""
import ctypes
import os

import numpy as np
import pytest

from oracle import ert_oracle as O
from pygimli_gb300.data import DataContainerERT, createData, geometricFactors, grid_scheme_3d
from pygimli_gb300.mesh import Mesh, create_box_mesh_3d, create_para_mesh_2d

pytestmark = pytest.mark.gpu

TOL_MAT = 1e-12
TOL_POT = 1e-6
TOL_J = 1e-5


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    from pygimli_gb300 import build
    build.build()
    return t


FORMS = {"fp64": dict(precision="fp64"), "mixed": dict(precision="mixed"),
         "mixed-fsai": dict(precision="mixed", precond="fsai"),
         "learned": dict(precision="mixed", precond="learned"),
         "fp64-ic0": dict(precision="fp64", precond="ic0")}
WEIGHTS = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "pygimli_gb300", "weights")


def learned_weights(mesh):
    """Packaged network weights for the mesh's kind of matrix: line_2d for
    2-D meshes, box_3d for linear and box_3d_p2 for quadratic tetrahedra."""
    if mesh.dim() == 2:
        return os.path.join(WEIGHTS, "line_2d.npz")
    return os.path.join(WEIGHTS, "box_3d_p2.npz" if mesh.cells.shape[1] == 10 else "box_3d.npz")


def fop_for(mesh, data, k=None, w=None, form=None, **kw):
    from pygimli_gb300 import ERTModelling
    if form is not None:
        kw.update(FORMS[form])
        if kw.get("precond") == "learned":
            kw["weights"] = learned_weights(mesh)
    fop = ERTModelling(**kw)
    if k is not None:
        fop.setkValues(k)
        fop.setWeights(w)
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    return fop


def load_case(golden_dir, name):
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"],
                z["boundaries"], z["boundary_markers"], z["boundary_cells"])
    if int(z["p2"]) == 1:
        mesh = mesh.createP2()
    elif int(z["p2"]) == 2:
        mesh = mesh.createH2()
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", z["kfac"])
    return z, mesh, data


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("precision", list(FORMS))
@pytest.mark.parametrize("name", ["ert2d_small", "ert2d_pd_wa", "ert3d_small", "ert3d_p2_small", "ert2d_p2_small",
                                  "ert2d_h2_small", "ert3d_h2_small"])
def test_golden_parity(torch, golden_dir, name, precision):
    z, mesh, data = load_case(golden_dir, name)
    fop = fop_for(mesh, data, form=precision)
    assert np.array_equal(fop.kValues(), z["k"]) and np.array_equal(fop.weights(), z["w"])
    rp, ci = fop.pattern()
    assert np.array_equal(rp, z["rowptr"]) and np.array_equal(ci, z["colidx"])
    rhoa = fop.response(z["rho"])
    e_rhoa = float(np.max(np.abs(rhoa - z["rhoa"]) / z["rhoa"]))
    for j, ki in enumerate(z["kidx"]):
        assert rel(fop.matrix(ki, 0), z["S"][j]) <= TOL_MAT
        assert rel(fop.matrix(ki, 1), z["S1"][j]) <= TOL_MAT
    prim = fop.primaryPotentials()
    for j, ki in enumerate(z["kidx"]):
        assert rel(prim[ki], z["primary"][j]) <= TOL_MAT
    e_pot = rel(fop.subPotentials(), z["subpot"])
    jdt = "float64" if precision == "fp64" else "float32"
    J = fop.createJacobian(z["rho"], dtype=jdt).cpu().numpy().astype(np.float64)
    e_J = float(np.linalg.norm(J - z["J"]) / np.linalg.norm(z["J"]))
    print(f"{name} {precision}: rhoa {e_rhoa:.2e} potentials {e_pot:.2e} J({jdt}) {e_J:.2e} "
          f"iters {fop.stats()['iterations']} stalled {fop.stats()['stalled_columns']}")
    assert e_rhoa <= TOL_POT and e_pot <= TOL_POT and e_J <= TOL_J


def _c1_case(seed=1):
    xs = np.arange(41.0)
    mesh = create_para_mesh_2d(xs, para_dx=0.25, para_depth=10.0)
    data = createData(xs, "dd")
    data.set("k", geometricFactors(data, 2))
    rng = np.random.default_rng(seed)
    rho = np.exp(rng.uniform(np.log(50.0), np.log(200.0), mesh.cellCount()))
    c = mesh.cellCenters()
    rho[(np.abs(c[:, 0] - 12.0) < 3.0) & (c[:, 1] > -4.0) & (c[:, 1] < -1.0)] = 10.0
    rho[(np.abs(c[:, 0] - 28.0) < 3.0) & (c[:, 1] > -6.0) & (c[:, 1] < -2.0)] = 1000.0
    return mesh, data, rho


@pytest.mark.parametrize("precision", list(FORMS))
def test_2d_config_vs_oracle(torch, precision):
    """41 electrodes, 741 dipole-dipole data, ~3.6k nodes, 17 wavenumbers."""
    mesh, data, rho = _c1_case()
    fop = fop_for(mesh, data, form=precision)
    assert len(fop.kValues()) == 17
    rhoa = fop.response(rho)
    jdt = "float64" if precision == "fp64" else "float32"
    J = fop.createJacobian(rho, dtype=jdt).cpu().numpy().astype(np.float64)
    P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], fop.kValues(), fop.weights())
    rhoa_o, u = P.response(rho)
    J_o = P.jacobian(u, rho)
    e_r = float(np.max(np.abs(rhoa - rhoa_o) / rhoa_o))
    e_J = float(np.linalg.norm(J - J_o) / np.linalg.norm(J_o))
    print(f"2d config {precision}: rhoa {e_r:.2e} J {e_J:.2e} iters {fop.stats()['iterations']} "
          f"stalled {fop.stats()['stalled_columns']}")
    assert e_r <= TOL_POT and e_J <= TOL_J


def _small_3d(nx=5, ny=4):
    e = np.array([(x, y) for x in np.arange(nx) * 4.0 for y in np.arange(ny) * 4.0])
    mesh = create_box_mesh_3d(e, h=2.0, para_margin=(2, 2), para_depth=8.0, outer=80.0, growth=1.8,
                              depth_growth=1.3)
    data = DataContainerERT(np.column_stack([e, np.zeros(len(e))]), grid_scheme_3d(nx, ny, 2))
    data.set("k", geometricFactors(data, 3))
    rng = np.random.default_rng(3)
    rho = np.exp(rng.normal(np.log(100.0), 1.0, mesh.cellCount()))
    return mesh, data, rho


@pytest.mark.parametrize("precision", list(FORMS))
def test_3d_vs_oracle(torch, precision):
    mesh, data, rho = _small_3d()
    fop = fop_for(mesh, data, form=precision)
    rhoa = fop.response(rho)
    jdt = "float64" if precision == "fp64" else "float32"
    J = fop.createJacobian(rho, dtype=jdt).cpu().numpy().astype(np.float64)
    P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], fop.kValues(), fop.weights())
    rhoa_o, u = P.response(rho)
    J_o = P.jacobian(u, rho)
    e_r = float(np.max(np.abs(rhoa - rhoa_o) / rhoa_o))
    e_J = float(np.linalg.norm(J - J_o) / np.linalg.norm(J_o))
    print(f"3d small {precision} ({mesh.nodeCount()} nodes): rhoa {e_r:.2e} J {e_J:.2e} "
          f"iters {fop.stats()['iterations']}")
    assert e_r <= TOL_POT and e_J <= TOL_J


def test_markers_shared_by_cells(torch):
    """Parameters spanning several cells and marker -1 cells prolongated."""
    mesh, data, rho = _c1_case(seed=2)
    mk = np.arange(mesh.cellCount()) // 4
    mk[::11] = -1
    mk[mk >= 0] = np.unique(mk[mk >= 0], return_inverse=True)[1]
    mesh.setCellMarkers(mk)
    model = np.exp(np.random.default_rng(4).uniform(np.log(30.0), np.log(300.0), int(mk.max()) + 1))
    fop = fop_for(mesh, data)
    rhoa = fop.response(model)
    J = fop.createJacobian(model).cpu().numpy()
    assert J.shape == (data.size(), int(mk.max()) + 1)
    rho_cell = O.map_model(mesh, model)
    P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], fop.kValues(), fop.weights())
    rhoa_o, u = P.response(rho_cell)
    J_o = P.jacobian(u, model)
    assert float(np.max(np.abs(rhoa - rhoa_o) / rhoa_o)) <= TOL_POT
    assert float(np.linalg.norm(J - J_o) / np.linalg.norm(J_o)) <= TOL_J


def test_fp32_jacobian_and_host_abi(torch, golden_dir):
    from pygimli_gb300 import _native
    z, mesh, data = load_case(golden_dir, "ert2d_small")
    fop = fop_for(mesh, data)
    r_dev = fop.response(z["rho"])
    J64 = fop.createJacobian(z["rho"]).cpu().numpy()
    J32 = fop.createJacobian(z["rho"], dtype="float32").cpu().numpy()
    assert np.linalg.norm(J32 - J64) <= TOL_J * np.linalg.norm(J64)
    L = _native.load()
    rho = np.ascontiguousarray(z["rho"])
    out = np.zeros(data.size())
    _native.check(fop._ctx, L.ertgb_response_host(fop._ctx, rho.ctypes.data_as(ctypes.c_void_p),
                                                  out.ctypes.data_as(ctypes.c_void_p)))
    assert np.array_equal(out, r_dev)
    Jh = np.zeros_like(J64)
    _native.check(fop._ctx, L.ertgb_jacobian_host(fop._ctx, rho.ctypes.data_as(ctypes.c_void_p), len(rho),
                                                  Jh.ctypes.data_as(ctypes.c_void_p), 0))
    assert np.array_equal(Jh, J64)


def test_error_paths(torch, golden_dir):
    from pygimli_gb300._native import NOT_CONVERGED, STATE, BAD_INPUT, ErtgbError
    z, mesh, data = load_case(golden_dir, "ert2d_small")
    fop = fop_for(mesh, data)
    # the C ABI refuses a Jacobian without potentials (ERTModelling.createJacobian
    # then computes them as the reference does, tests/test_jacobian_first.py)
    J = torch.empty((data.size(), mesh.cellCount()), dtype=torch.float64, device="cuda")
    rc = fop._lib.ertgb_jacobian(fop._ctx, None, 0, ctypes.c_void_p(J.data_ptr()), 0, None)
    assert rc == STATE
    bad = z["rho"].copy()
    bad[5] = 0.0
    with pytest.raises(ValueError):
        fop.response(bad)
    dev = torch.tensor(bad, device="cuda")
    dev[7] = -1.0
    with pytest.raises(ErtgbError) as e:
        fop.response(dev)
    assert e.value.code == BAD_INPUT
    fop.setSolverTolerance(1e-10, 1)
    with pytest.raises(ErtgbError) as e:
        fop.response(z["rho"])
    assert e.value.code == NOT_CONVERGED
    fop.setSolverTolerance(1e-10, 20000)
    r = fop.response(z["rho"])
    assert np.max(np.abs(r - z["rhoa"]) / z["rhoa"]) <= TOL_POT


@pytest.mark.parametrize("name", ["ert2d_h2_small", "ert3d_h2_small"])
def test_forward_mesh_refinement(torch, golden_dir, name):
    """setMesh(parameter mesh) solves on its H2 refinement (the default of
    pyGIMLi's mesh-based modelling) with one parameter per parent cell."""
    from pygimli_gb300 import ERTModelling
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    para = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"],
                z["boundaries"], z["boundary_markers"], z["boundary_cells"])
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", z["kfac"])
    fop = ERTModelling(precision="mixed", precond="fsai")
    fop.setData(data)
    fop.setMesh(para)
    # one region per cell marker: the lowest became background; make every
    # cell a parameter again, as the fixture's reference run has it
    fop.setRegionProperties(int(para.cell_markers.min()), background=False)
    assert fop.mesh().cellCount() == para.cellCount() * (4 if para.dim() == 2 else 8)
    assert fop.parameterCount == para.cellCount()
    rhoa = fop.response(z["rho"])
    assert float(np.max(np.abs(rhoa - z["rhoa"]) / z["rhoa"])) <= TOL_POT
    J = fop.createJacobian(z["rho"]).cpu().numpy()
    assert J.shape == z["J"].shape
    assert float(np.linalg.norm(J - z["J"]) / np.linalg.norm(z["J"])) <= TOL_J


def _jacobian_rows_from_potentials(mesh, data, k, w, u, model, rows):
    K, M = O.element_matrices(mesh.dim(), mesh.nodes, mesh.cells)
    ab = data.abmn()[rows]
    out = np.zeros((len(rows), mesh.cellCount()))
    cells = mesh.cells
    for ki in range(len(k)):
        S = M * (k[ki] ** 2) + K
        Uc = np.transpose(u[ki][:, cells], (1, 2, 0))
        Uc = np.concatenate([Uc, np.zeros(Uc.shape[:2] + (1,))], axis=2)
        V = np.einsum("cij,cje->cie", S, Uc)
        dab = V[:, :, ab[:, 0]] - V[:, :, ab[:, 1]]
        dmn = Uc[:, :, ab[:, 2]] - Uc[:, :, ab[:, 3]]
        out += w[ki] * np.einsum("cid,cid->dc", dab, dmn)
    kf = data["k"][rows]
    return out / ((model ** 2)[None, :] / kf[:, None])


def test_3d_config_properties(torch):
    """96 electrodes on 12 x 8, ~88k nodes, ~486k tetrahedra, 5336 data."""
    e = np.array([(x, y) for x in np.arange(12) * 4.0 for y in np.arange(8) * 4.0])
    mesh = create_box_mesh_3d(e)
    data = DataContainerERT(np.column_stack([e, np.zeros(len(e))]), grid_scheme_3d(12, 8))
    data.set("k", geometricFactors(data, 3))
    rng = np.random.default_rng(7)
    rho = np.exp(rng.normal(np.log(100.0), 1.0, mesh.cellCount()))
    fop = fop_for(mesh, data)
    r1 = fop.response(rho)
    st = fop.stats()
    # linearity in the resistivity scale
    r2 = fop.response(2.0 * rho)
    assert float(np.max(np.abs(r2 - 2.0 * r1) / (2.0 * r1))) <= TOL_POT
    # Jacobian rows against a recomputation from the GPU potentials
    J = fop.createJacobian(2.0 * rho)
    rows = np.array([0, 17, 600, 1500, 2500, 4000, 5300])
    Jr = J[torch.as_tensor(rows, device=J.device)].cpu().numpy()
    u = fop.subPotentials()
    Jo = _jacobian_rows_from_potentials(mesh, data, fop.kValues(), fop.weights(), u, 2.0 * rho, rows)
    assert float(np.linalg.norm(Jr - Jo) / np.linalg.norm(Jo)) <= TOL_J
    # FP32 Jacobian (FP64 differences) against the same rows
    J32 = fop.createJacobian(2.0 * rho, dtype="float32")
    J32r = J32[torch.as_tensor(rows, device=J32.device)].cpu().numpy().astype(np.float64)
    assert float(np.linalg.norm(J32r - Jo) / np.linalg.norm(Jo)) <= TOL_J
    del J, J32
    # mixed-precision solves (Jacobi and FSAI) reach the same answer
    fop.setPrecision("mixed")
    r3 = fop.response(2.0 * rho)
    st3 = fop.stats()
    assert float(np.max(np.abs(r3 - r2) / r2)) <= TOL_POT
    fop.setPreconditioner("fsai")
    r4 = fop.response(2.0 * rho)
    st4 = fop.stats()
    assert float(np.max(np.abs(r4 - r2) / r2)) <= TOL_POT
    fop.setPreconditioner("jacobi")
    fop.setPrecision("fp64")
    print(f"3d config: mixed iters {st3['iterations']} solve {st3['ms_solve']:.1f} ms; mixed+fsai iters "
          f"{st4['iterations']} solve {st4['ms_solve']:.1f} ms")
    # homogeneous half-space: apparent resistivity equals the resistivity
    rh = fop.response(np.full(mesh.cellCount(), 100.0))
    assert float(np.max(np.abs(rh - 100.0) / 100.0)) < 0.05
    print(f"3d config: iters {st['iterations']} solve {st['ms_solve']:.1f} ms, homogeneous "
          f"max dev {np.max(np.abs(rh - 100.0)):.3f}")


def test_jacobian_data_chunks(torch):
    """A scheme whose distinct current and potential dipoles (about 9,900)
    make one cell's FP64 dipole tables exceed shared memory: the Jacobian is
    built in data chunks, each with its own dipole tables; rows are checked
    against the oracle's rows recomputed from the GPU potentials."""
    e = np.array([(x, y) for x in np.arange(10) * 2.0 for y in np.arange(10) * 2.0])
    mesh = create_box_mesh_3d(e, h=2.0, para_margin=(1, 1), para_depth=4.0, outer=60.0, growth=2.0,
                              depth_growth=1.6)
    pairs = [(a, b) for a in range(100) for b in range(a + 1, 100)]
    npair = len(pairs)
    ab = np.array([pairs[i % npair] + pairs[(7 * i + 3) % npair] for i in range(5000)], np.int32)
    ab = ab[(ab[:, 0] != ab[:, 2]) & (ab[:, 0] != ab[:, 3]) & (ab[:, 1] != ab[:, 2]) & (ab[:, 1] != ab[:, 3])]
    data = DataContainerERT(np.column_stack([e, np.zeros(len(e))]), ab)
    with np.errstate(divide="ignore"):
        kf = geometricFactors(data, 3)
    ok = np.isfinite(kf) & (np.abs(kf) < 1e6)  # drop symmetric configurations (no signal)
    data = DataContainerERT(np.column_stack([e, np.zeros(len(e))]), ab[ok])
    data.set("k", kf[ok])
    rng = np.random.default_rng(5)
    rho = np.exp(rng.normal(np.log(100.0), 0.7, mesh.cellCount()))
    fop = fop_for(mesh, data)
    fop.response(rho)
    J = fop.createJacobian(rho)
    rows = np.array([0, 1, 999, 2500, data.size() - 1])
    Jr = J[torch.as_tensor(rows, device=J.device)].cpu().numpy()
    Jo = _jacobian_rows_from_potentials(mesh, data, fop.kValues(), fop.weights(), fop.subPotentials(), rho, rows)
    assert float(np.linalg.norm(Jr - Jo) / np.linalg.norm(Jo)) <= TOL_J


def _spmm_case(golden_dir, torch, seed=0, ld=64):
    """Golden system matrices of three wavenumbers as one multi-matrix
    operator, 11 columns per matrix (33 used, padded to 64)."""
    z = np.load(os.path.join(golden_dir, "ert2d_small.npz"))
    rp, ci, vals = z["rowptr"], z["colidx"], z["S"]
    n, nnz = len(rp) - 1, len(ci)
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, ld))
    dev = torch.device("cuda")
    t = {"rp": torch.from_numpy(rp.astype(np.int32)).to(dev), "ci": torch.from_numpy(ci.astype(np.int32)).to(dev),
         "v": torch.from_numpy(np.ascontiguousarray(vals)).to(dev), "X": torch.from_numpy(X).to(dev)}
    import scipy.sparse as sp
    Y = np.zeros((n, ld))
    for col in range(ld):
        kk = min(col // 11, 2)
        Y[:, col] = sp.csr_matrix((vals[kk], ci, rp), shape=(n, n)) @ X[:, col]
    return n, nnz, t, X, Y, np.einsum("ij,ij->j", X, Y)


def _call_spmm(fn, n, nnz, t, ld, torch):
    Y = torch.empty((n, ld), dtype=torch.float64, device="cuda")
    dots = torch.empty(ld, dtype=torch.float64, device="cuda")
    vp = ctypes.c_void_p
    rc = fn(n, nnz, vp(t["rp"].data_ptr()), vp(t["ci"].data_ptr()), vp(t["v"].data_ptr()), 3, 11, ld,
            vp(t["X"].data_ptr()), vp(Y.data_ptr()), vp(dots.data_ptr()), vp(torch.cuda.current_stream().cuda_stream))
    return rc, Y, dots


def test_csr_spmm_dot_entry(torch, golden_dir):
    from pygimli_gb300 import _native
    L = _native.load()
    n, nnz, t, X, Y_ref, d_ref = _spmm_case(golden_dir, torch)
    rc, Y, dots = _call_spmm(L.ertgb_csr_spmm_dot, n, nnz, t, 64, torch)
    _native.check(None, rc)
    torch.cuda.synchronize()
    assert rel(Y.cpu().numpy(), Y_ref) <= TOL_MAT
    assert rel(dots.cpu().numpy(), d_ref) <= TOL_MAT
    rc, _, _ = _call_spmm(L.ertgb_csr_spmm_dot, n, nnz, t, 48, torch)
    assert rc == _native.BAD_INPUT and b"multiple of 32" in L.ertgb_last_error(None)


@pytest.mark.parametrize("name", ["mesh2d", "mesh3d_p2"])
def test_files_to_response(torch, name, tmp_path):
    """Mesh from the reference's binary mesh file (every facet a boundary,
    outer facets with only a right cell) and data through the unified data
    format: the GPU response and Jacobian equal the oracle's on that mesh."""
    io = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "io", "expected")
    mesh = Mesh.load(os.path.join(io, name + ".bms"))
    if mesh.dim() == 2:
        d0 = createData(np.arange(4.0), "dd")
        d0.set("k", geometricFactors(d0, 2))
    else:
        d0 = DataContainerERT(np.array([[0.0, 0.0, 0.0], [2.0, 0.0, 0.0]]),
                              np.array([[0, -1, 1, -1], [1, -1, 0, -1]]))
        d0.set("k", geometricFactors(d0, 3))
    f = tmp_path / "scheme.dat"
    d0.save(str(f), "a b m n k")
    data = DataContainerERT(str(f))
    assert np.array_equal(data.abmn(), d0.abmn())
    rho = 20.0 + (np.arange(mesh.cellCount()) % 5) * 15.0
    fop = fop_for(mesh, data)
    rhoa = fop.response(rho)
    J = fop.createJacobian(rho).cpu().numpy()
    P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], fop.kValues(), fop.weights())
    rhoa_o, u = P.response(rho)
    J_o = P.jacobian(u, rho)
    assert rel(rhoa, rhoa_o) <= TOL_POT
    assert np.linalg.norm(J - J_o) / np.linalg.norm(J_o) <= TOL_J


@pytest.mark.parametrize("dim", [2, 3])
def test_region_manager_forward(torch, dim):
    """setMesh(mesh) with region markers (1 outside, 2 parameter box, 3 and 4
    blocks): region 1 becomes background (filled from its neighbours),
    region 3 is fixed, region 4 single; response and Jacobian over the
    renumbered parameters equal the oracle's on the same forward mesh."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_regions_golden import region_mesh
    from pygimli_gb300 import ERTModelling
    m = region_mesh(dim)
    if dim == 2:
        data = createData(np.arange(9.0), "dd")
    else:
        e = np.array([(x, y, 0.0) for x in (0.0, 2.0, 4.0) for y in (0.0, 2.0)])
        data = DataContainerERT(e, np.array([[0, 1, 2, 3], [0, 2, 4, 5], [1, 3, 0, 5], [2, 4, 1, 3]]))
    data.set("k", geometricFactors(data, dim))
    fop = ERTModelling()
    fop.setData(data)
    fop.setMesh(m)
    P0 = fop.parameterCount
    fop.setDefaultBackground()  # setMesh applied it already
    assert fop.parameterCount == P0
    fop.setRegionProperties(3, fix=50.0)
    fop.setRegionProperties(4, single=True)
    P = fop.parameterCount
    assert P == fop.regionManager().parameterCount()
    model = np.linspace(20.0, 200.0, P)
    rhoa = fop.response(model)
    J = fop.createJacobian(model).cpu().numpy()
    fwd = fop.mesh()
    att = fop.mapERTModel(model)
    Po = O.Problem(fwd, data.sensorPositions(), data.abmn(), data["k"], fop.kValues(), fop.weights())
    rhoa_o, u = Po.response(att)
    J_o = Po.jacobian(u, model, n_params=P)
    assert J.shape == (data.size(), P)
    assert rel(rhoa, rhoa_o) <= TOL_POT
    assert np.linalg.norm(J - J_o) / np.linalg.norm(J_o) <= TOL_J


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["ert2d_complex_small", "ert3d_complex_small"])
def test_complex_resistivity_golden(torch, golden_dir, name, precision):
    """setComplex(True): complex apparent resistivities and the complex
    Jacobian equal the reference's own complex path (total potential,
    complex symmetric systems) on its fixtures; the GPU solves with block
    COCG to rtol 1e-10 where the reference factors."""
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"],
                z["boundaries"], z["boundary_markers"], z["boundary_cells"])
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", z["kfac"])
    fop = fop_for(mesh, data, z["k"], z["w"], form=precision)
    fop.setComplex(True)
    assert fop.parameterCount == 2 * mesh.cellCount()
    rho = z["rho"]
    out = fop.response(np.concatenate([rho.real, rho.imag]))
    D = data.size()
    rhoa = out[:D] + 1j * out[D:]
    e_r = float(np.max(np.abs(rhoa - z["rhoa"]) / np.abs(z["rhoa"])))
    J = fop.createJacobian(rho).cpu().numpy()
    e_j = float(np.linalg.norm(J - z["J"]) / np.linalg.norm(z["J"]))
    st = fop.stats()
    print(f"{name} {precision}: rhoa {e_r:.2e} J {e_j:.2e} COCG iterations {st['iterations']}, "
          f"columns finished in FP64 {st['stalled_columns']}")
    assert J.shape == z["J"].shape
    assert e_r <= 1e-7 and e_j <= 1e-6


def test_complex_flip_convention(torch, golden_dir):
    """A complex start model from data whose median imaginary part is
    negative flips it to positive (ertModelling.py:168-186); response and
    createJacobian then take and return that convention (:204-238):
    response(flip(m)) = flip(response(m)) and the Jacobian conjugated, bit
    for bit (the same deterministic solves)."""
    z = np.load(os.path.join(golden_dir, "ert2d_complex_small.npz"))
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"],
                z["boundaries"], z["boundary_markers"], z["boundary_cells"])
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", z["kfac"])
    fop = fop_for(mesh, data, z["k"], z["w"], form="fp64")
    fop.setComplex(True)
    rho = z["rho"]
    m = np.concatenate([rho.real, rho.imag])
    r0 = fop.response(m)
    J0 = fop.createJacobian(rho).cpu().numpy()
    D = data.size()
    sm = fop.createStartModel(np.concatenate([np.abs(r0[:D]), -np.abs(r0[D:]) - 1.0]))
    P = mesh.cellCount()
    assert fop._conjImag and np.all(sm[P:] > 0) and len(sm) == 2 * P
    r1 = fop.response(fop.flipImagPart(m))
    assert np.array_equal(r1, fop.flipImagPart(r0))
    J1 = fop.createJacobian(np.conj(rho)).cpu().numpy()
    assert np.array_equal(J1, np.conj(J0))


def test_complex_sign_and_mirror_symmetry(torch):
    """The reference's complex simulate test (pygimli/testing/
    test_ERTManager_simulate.py) on this operator: layered complex
    resistivity (99.595 + 8.987j above -5 m, 59.595 + 8.987j below), five
    electrodes; a configuration and its copy with the sign of k reversed give
    the same complex apparent resistivity, its mirror image the same up to
    the mesh's asymmetry, and phases and amplitudes are positive."""
    from pygimli_gb300 import ERTModelling
    xs = np.arange(-2.0, 3.0)
    mesh = create_para_mesh_2d(xs, para_dx=0.25, para_depth=8.0)
    data = DataContainerERT(np.column_stack([xs, np.zeros(5), np.zeros(5)]),
                            np.array([[0, 1, 3, 2], [0, 1, 2, 3], [3, 2, 1, 0]]))
    data.set("k", geometricFactors(data, 2))
    assert np.isclose(data["k"][0], -data["k"][1], rtol=1e-14)
    depth = mesh.cellCenters()[:, 1]
    rho = np.where(depth > -5.0, 99.595 + 8.987j, 59.595 + 8.987j)
    for precision in ("fp64", "mixed"):
        fop = ERTModelling(precision=precision)
        fop.setData(data)
        fop.setMesh(mesh, ignoreRegionManager=True)
        fop.setComplex(True)
        out = fop.response(rho)
        z = out[:3] + 1j * out[3:]
        assert abs(z[1] - z[0]) / abs(z[0]) < 1e-9, z
        assert abs(z[2] - z[0]) / abs(z[0]) < 2e-2, z
        assert np.all(np.abs(z) > 0) and np.all(np.angle(z) > 0), z


def test_simulate_forms(torch):
    """simulate() as pg.physics.ert.simulate: a resistivity map by marker, a
    per-cell array and N rows agree; rhoa scales with the model; complex maps
    give positive phases; seeded noise is reproducible and uses
    estimateError's errors; u = rhoa / k at 1 A."""
    from pygimli_gb300 import simulate
    from pygimli_gb300.data import estimateError
    xs = np.arange(8.0)
    mesh = create_para_mesh_2d(xs, para_dx=0.5, para_depth=4.0)
    mk = np.where(mesh.cellCenters()[:, 1] > -1.5, 1, 2).astype(np.int32)
    mesh.setCellMarkers(mk)
    scheme = createData(xs, "dd")
    d = simulate(mesh, scheme, [[1, 100.0], [2, 10.0]])
    assert np.all(d["rhoa"] > 0) and d.allNonZero("k")
    assert np.allclose(d["u"], d["rhoa"] / d["k"]) and np.all(d["i"] == 1.0)
    rho = np.where(mk == 1, 100.0, 10.0)
    a = simulate(mesh, scheme, rho, returnArray=True)
    rows = simulate(mesh, scheme, np.vstack([rho, 2.0 * rho]), returnArray=True)
    assert np.allclose(a, d["rhoa"], rtol=1e-12) and rows.shape == (2, scheme.size())
    assert np.allclose(rows[1], 2.0 * rows[0], rtol=1e-8)
    c = simulate(mesh, scheme, [[1, 100.0 + 1.0j], [2, 10.0 + 0.5j]])
    assert np.all(c["rhoa"] > 0) and np.all(c["phia"] > 0)
    n1 = simulate(mesh, scheme, rho, noiseLevel=0.03, seed=5)
    n2 = simulate(mesh, scheme, rho, noiseLevel=0.03, seed=5)
    assert np.array_equal(n1["rhoa"], n2["rhoa"]) and not np.allclose(n1["rhoa"], a)
    ref = d.copy()
    for t in ("u", "i", "r"):
        ref.set(t, np.zeros(ref.size()))
    assert np.allclose(n1["err"], estimateError(ref, relativeError=0.03, absoluteUError=1e-4, absoluteCurrent=1))
