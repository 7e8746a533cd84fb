"""The oracle (oracle/ert_oracle.py) against the reference's own outputs.

The fixtures in tests/golden/ were produced by running the reference's C++
ERT code (built from its sources, see tests/golden/make_golden.py).  These
CPU tests pin the numpy restatement that the GPU parity tests use as the
checker, and the host-side restatements of the package (quadrature,
electrode search, geometric factors)."""
import os

import numpy as np
import pytest

from oracle import ert_oracle as O
from pygimli_gb300.data import DataContainerERT, geometricFactors
from pygimli_gb300.ert import search_electrodes, surface_info
from pygimli_gb300.kwave import gauss_laguerre, gauss_legendre, init_kwave_list
from pygimli_gb300.mesh import Mesh

CASES = ["ert2d_small", "ert2d_pd_wa", "ert3d_small", "ert3d_p2_small", "ert2d_p2_small", "ert2d_h2_small",
         "ert3d_h2_small"]


def load_case(golden_dir, name):
    """Mesh of a fixture: the stored P1 mesh, refined with create_p2 / create_h2
    for the refined cases (the reference ran its own Mesh::createP2 /
    Mesh::createH2)."""
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"],
                z["boundaries"], z["boundary_markers"], z["boundary_cells"])
    if int(z["p2"]) == 1:
        mesh = mesh.createP2()
    elif int(z["p2"]) == 2:
        mesh = mesh.createH2()
    return z, mesh


@pytest.mark.parametrize("name", ["ert3d_p2_small", "ert2d_p2_small", "ert2d_h2_small", "ert3d_h2_small"])
def test_refinement_matches_reference(golden_dir, name):
    z, mesh = load_case(golden_dir, name)
    assert np.array_equal(mesh.nodes, z["ref_nodes"])
    assert np.array_equal(mesh.cells, z["ref_cells"])
    assert np.array_equal(mesh.node_markers, z["ref_node_markers"])
    assert np.array_equal(mesh.cell_markers, z["ref_cell_markers"])
    assert np.array_equal(mesh.boundaries, z["ref_boundaries"])
    assert np.array_equal(mesh.boundary_markers, z["ref_boundary_markers"])


def test_bessel_matches_reference(golden_dir):
    z = np.load(os.path.join(golden_dir, "bessel_quadrature.npz"))
    k0 = O.besselK0(z["x"])
    k1 = O.besselK1(z["x"])
    assert np.max(np.abs(k0 - z["k0"]) / np.abs(z["k0"])) < 1e-15
    assert np.max(np.abs(k1 - z["k1"]) / np.abs(z["k1"])) < 1e-15


@pytest.mark.parametrize("n", [4, 5, 8, 12, 17, 21])
def test_quadrature_matches_reference(golden_dir, n):
    z = np.load(os.path.join(golden_dir, "bessel_quadrature.npz"))
    x, w = gauss_legendre(0.0, 1.0, n)
    assert np.array_equal(x, z[f"leg_x_{n}"]) and np.array_equal(w, z[f"leg_w_{n}"])
    x, w = gauss_laguerre(n)
    assert np.array_equal(x, z[f"lag_x_{n}"]) and np.array_equal(w, z[f"lag_w_{n}"])


@pytest.mark.parametrize("name", CASES)
def test_host_setup_matches_reference(golden_dir, name):
    z, mesh = load_case(golden_dir, name)
    k, w = init_kwave_list(mesh.dim(), z["sensors"])
    assert np.array_equal(k, z["k"]) and np.array_equal(w, z["w"])
    assert np.array_equal(search_electrodes(mesh, z["sensors"]).nodes, z["electrode_nodes"])
    d = DataContainerERT(z["sensors"], z["abmn"])
    kf = geometricFactors(d, mesh.dim())
    assert np.max(np.abs(kf - z["kfac_ref"]) / np.abs(z["kfac_ref"])) < 1e-14
    sz, topo = surface_info(mesh)
    assert sz == 0.0 and not topo


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(golden_dir, name):
    z, mesh = load_case(golden_dir, name)
    P = O.Problem(mesh, z["sensors"], z["abmn"], z["kfac"], z["k"], z["w"])
    # CSR pattern: bit-exact
    assert np.array_equal(P.rowptr, z["rowptr"]) and np.array_equal(P.cols, z["colidx"])
    rho = z["rho"]
    rho_cell = O.map_model(mesh, rho)
    for j, ki in enumerate(z["kidx"]):
        S = P.assemble(rho_cell, ki)
        S1 = P.assemble(np.ones_like(rho_cell), ki)
        assert np.max(np.abs(S - z["S"][j])) <= 1e-12 * np.max(np.abs(z["S"][j]))
        assert np.max(np.abs(S1 - z["S1"][j])) <= 1e-12 * np.max(np.abs(z["S1"][j]))
        assert np.max(np.abs(P.up[ki] - z["primary"][j])) <= 1e-13 * np.max(np.abs(z["primary"][j]))
    rhoa, u = P.response(rho_cell)
    assert np.max(np.abs(rhoa - z["rhoa"]) / z["rhoa"]) < 1e-10
    assert np.max(np.abs(u - z["subpot"])) <= 1e-10 * np.max(np.abs(z["subpot"]))
    J = P.jacobian(u, rho)
    assert np.linalg.norm(J - z["J"]) <= 1e-10 * np.linalg.norm(z["J"])


def test_oracle_model_mapping_prolongation(golden_dir):
    """Marker -1 cells are filled from their neighbours (mesh.cpp:2247-2316)."""
    from pygimli_gb300.modelmap import map_model
    z, mesh = load_case(golden_dir, "ert2d_small")
    mk = mesh.cell_markers.copy()
    mk[::7] = -1
    mk[mk >= 0] = np.arange(np.sum(mk >= 0))
    mesh.setCellMarkers(mk)
    model = np.linspace(10.0, 100.0, int(mk.max()) + 1)
    a = O.map_model(mesh, model)
    b = map_model(mesh, model)
    assert np.all(a > 0) and np.allclose(a, b, rtol=1e-14, atol=0)
    c = map_model(mesh, model, background=42.0)
    assert np.all(c[mk == -1] == 42.0)


@pytest.mark.parametrize("name", ["ert2d_complex_small", "ert3d_complex_small"])
def test_complex_oracle_matches_reference(golden_dir, name):
    """Complex resistivity: the oracle's total-potential restatement equals
    the reference's own complex path (setComplex(true)) to rounding."""
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"],
                z["boundaries"], z["boundary_markers"], z["boundary_cells"])
    P = O.Problem(mesh, z["sensors"], z["abmn"], z["kfac"], z["k"], z["w"])
    r, u = P.response_complex(z["rho"])
    assert np.max(np.abs(r - z["rhoa"]) / np.abs(z["rhoa"])) < 1e-12
    J = P.jacobian_complex(u, z["rho"])
    assert np.linalg.norm(J - z["J"]) / np.linalg.norm(z["J"]) < 1e-12
