"""Generate the golden fixtures of tests/golden/ by running the reference's own
C++ ERT modelling code (built from the reference sources by oracle/Makefile
into oracle/_ref/libgimli_ref.so and driven through oracle/ref_driver.py).

Run from the repository root after ``make -C oracle``:

    python tests/golden/make_golden.py [fixture names ...]

(no names: all fixtures).
Each fixture holds the inputs (mesh arrays, sensors, ABMN, geometric
factors, resistivity) and the reference outputs: wavenumbers/weights, the
assembled system matrices (CSR), primary potentials, sub-potentials,
apparent resistivities and the Jacobian.  Sizes are kept small so the
fixtures stay a few hundred KB.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle.ref_driver import RefModelling, besselK0, besselK1, lib  # noqa: E402
from pygimli_gb300.data import DataContainerERT, createData, geometricFactors, grid_line_scheme  # noqa: E402
from pygimli_gb300.mesh import create_box_mesh_3d, create_para_mesh_2d  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def _resistivity(mesh, seed):
    rng = np.random.default_rng(seed)
    rho = np.exp(rng.uniform(np.log(50.0), np.log(200.0), mesh.cellCount()))
    c = mesh.cellCenters()
    d = mesh.dim() - 1
    box = (np.abs(c[:, 0] - c[:, 0].mean() * 0.5) < 2.0) & (c[:, d] > -2.0)
    rho[box] = 10.0
    return rho


def case(name, mesh, data, seed, threads=1, p2=False, h2=False):
    """One fixture.  With p2 / h2 the reference refines the given mesh itself
    (Mesh::createP2 / Mesh::createH2); the resistivity stays one value per
    cell of the given mesh and reaches the refined cells through their
    markers (the parent's cell index)."""
    if only and name not in only:
        return
    R = RefModelling(mesh, data.sensorPositions(), data.abmn(), data["k"], threads=threads,
                     keep_matrices=True, p2=p2, h2=h2)
    k, w = R.kw()
    rho = _resistivity(mesh, seed)
    rhoa = R.response(rho)
    mats = R.matrices
    sub = R.subpotentials()
    sub = sub.reshape(len(k), data.sensorCount(), -1)
    J = R.jacobian(rho)
    kidx = np.unique([0, len(k) // 2, len(k) - 1])
    prim = np.stack([np.stack([R.primary(e, k[i], 0.0) for e in range(data.sensorCount())]) for i in kidx])
    rp = np.stack([mats[i][0] for i in kidx])
    ci = np.stack([mats[i][1] for i in kidx])
    va = np.stack([mats[i][2] for i in kidx])
    xyz_r, nm_r, cells_r, cm_r, bnd_r, bm_r = R.mesh_arrays()
    rho1 = np.ones(len(cells_r))
    src_center = xyz_r[R.electrode_nodes()].mean(axis=0)
    # boundaries of the refined mesh: the reference appends the new ones
    # after those created from the input boundaries
    nb_r = mesh.boundaryCount() * (1 if not h2 else (4 if mesh.dim() == 3 else 2))
    S1 = np.stack([R.assemble(rho1, k[i], src_center)[2] for i in kidx])
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"),
        dim=mesh.dim(), nodes=mesh.nodes, cells=mesh.cells, cell_markers=mesh.cell_markers,
        node_markers=mesh.node_markers, boundaries=mesh.boundaries,
        boundary_markers=mesh.boundary_markers, boundary_cells=mesh.boundary_cells,
        sensors=data.sensorPositions(), abmn=data.abmn(), kfac=data["k"],
        kfac_ref=R.geometric_factors(), rho=rho, k=k, w=w, rhoa=rhoa,
        electrode_nodes=R.electrode_nodes(), kidx=kidx, rowptr=rp[0], colidx=ci[0], S=va, S1=S1,
        primary=prim, subpot=sub, J=J, p2=2 if h2 else int(p2), ref_nodes=xyz_r, ref_cells=cells_r,
        ref_node_markers=nm_r, ref_cell_markers=cm_r, ref_boundaries=bnd_r[:nb_r],
        ref_boundary_markers=bm_r[:nb_r])
    R.close()
    print(name, mesh, len(data), "k:", len(k), "J:", J.shape)


def case_complex(name, mesh, data, seed):
    """Complex resistivity (setComplex(true): the reference's total-potential
    path with complex symmetric matrices): per-cell complex resistivity of
    amplitude 50-200 Ohm m and phase -5 to -30 mrad (one value per cell
    marker), complex apparent resistivities and the complex Jacobian."""
    if only and name not in only:
        return
    R = RefModelling(mesh, data.sensorPositions(), data.abmn(), data["k"])
    k, w = R.kw()
    rng = np.random.default_rng(seed)
    C = mesh.cellCount()
    rho_c = np.exp(rng.uniform(np.log(50.0), np.log(200.0), C)) * np.exp(-1j * rng.uniform(0.005, 0.03, C))
    rhoa = R.response_complex(rho_c.real, rho_c.imag)
    J = R.jacobian_complex(rho_c.real, rho_c.imag)
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"),
        dim=mesh.dim(), nodes=mesh.nodes, cells=mesh.cells, cell_markers=mesh.cell_markers,
        node_markers=mesh.node_markers, boundaries=mesh.boundaries,
        boundary_markers=mesh.boundary_markers, boundary_cells=mesh.boundary_cells,
        sensors=data.sensorPositions(), abmn=data.abmn(), kfac=data["k"], k=k, w=w,
        rho=rho_c, rhoa=rhoa, J=J, p2=0)
    R.close()
    print(name, mesh, len(data), "k:", len(k), "J:", J.shape)


def bessel_table():
    x = np.concatenate([np.geomspace(1e-6, 2.0, 60), np.linspace(2.0, 40.0, 60), [2.0, 3.75, 50.0]])
    k0 = np.array([besselK0(v) for v in x])
    k1 = np.array([besselK1(v) for v in x])
    gl, gw, lx, lw = {}, {}, {}, {}
    import ctypes
    out = {}
    for n in (4, 5, 8, 12, 17, 21):
        a = np.zeros(n)
        b = np.zeros(n)
        lib().ref_gauss_legendre(n, a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p))
        out[f"leg_x_{n}"] = a.copy()
        out[f"leg_w_{n}"] = b.copy()
        lib().ref_gauss_laguerre(n, a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p))
        out[f"lag_x_{n}"] = a.copy()
        out[f"lag_w_{n}"] = b.copy()
    np.savez_compressed(os.path.join(OUT, "bessel_quadrature.npz"), x=x, k0=k0, k1=k1, **out)
    print("bessel_quadrature", len(x))


only = set(sys.argv[1:])


def main():
    if not only or "bessel_quadrature" in only:
        bessel_table()
    # 2.5-D: 11 electrodes, dipole-dipole
    xs = np.arange(11.0)
    m2 = create_para_mesh_2d(xs, para_dx=0.5, para_depth=4.0)
    d2 = createData(xs, "dd")
    d2["k"] = geometricFactors(d2, 2)
    case("ert2d_small", m2, d2, seed=11)
    # 2.5-D with pole-dipole (electrode at infinity) and Wenner
    d2b = createData(xs, "pd")
    wa = createData(xs, "wa").abmn()
    d2b = DataContainerERT(d2b.sensorPositions(), np.vstack([d2b.abmn(), wa]))
    d2b["k"] = geometricFactors(d2b, 2)
    case("ert2d_pd_wa", m2, d2b, seed=12)
    # 3-D: 4 x 3 electrode grid, dipole-dipole + pole-dipole lines
    e = np.array([(x, y) for x in np.arange(4) * 4.0 for y in np.arange(3) * 4.0])
    m3 = create_box_mesh_3d(e, h=2.0, para_margin=(2, 2), para_depth=6.0, outer=60.0,
                            growth=2.0, depth_growth=1.5)
    ab = np.vstack([grid_line_scheme((4, 3), "dd"), grid_line_scheme((4, 3), "pd")])
    d3 = DataContainerERT(np.column_stack([e, np.zeros(len(e))]), ab)
    d3["k"] = geometricFactors(d3, 3)
    case("ert3d_small", m3, d3, seed=13)
    # quadratic elements (the reference's Mesh::createP2 of the same meshes)
    m3p = create_box_mesh_3d(np.array([(x, y) for x in np.arange(3) * 4.0 for y in np.arange(2) * 4.0]),
                             h=2.0, para_margin=(1, 1), para_depth=4.0, outer=40.0, growth=2.2, depth_growth=1.6)
    e3p = np.array([(x, y) for x in np.arange(3) * 4.0 for y in np.arange(2) * 4.0])
    ab3p = np.vstack([grid_line_scheme((3, 2), "pd"), np.array([[0, 1, 2, 3], [0, 2, 4, 5]], np.int32)])
    d3p = DataContainerERT(np.column_stack([e3p, np.zeros(len(e3p))]), ab3p)
    d3p["k"] = geometricFactors(d3p, 3)
    case("ert3d_p2_small", m3p, d3p, seed=14, p2=True)
    xs7 = np.arange(7.0)
    m2p = create_para_mesh_2d(xs7, para_dx=1.0, para_depth=3.0)
    d2p = createData(xs7, "dd")
    d2p["k"] = geometricFactors(d2p, 2)
    case("ert2d_p2_small", m2p, d2p, seed=15, p2=True)
    # uniform refinement, the default forward mesh of pyGIMLi's mesh-based
    # modelling (one parameter per parent cell)
    case("ert2d_h2_small", m2p, d2p, seed=16, h2=True)
    case("ert3d_h2_small", m3p, d3p, seed=17, h2=True)
    # complex resistivity (induced polarisation)
    case_complex("ert2d_complex_small", m2p, d2p, seed=18)
    case_complex("ert3d_complex_small", m3p, d3p, seed=19)


if __name__ == "__main__":
    main()
