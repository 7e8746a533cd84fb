"""The banded direct solve (ERTModelling(precond="band"), FP64): the exact
Cholesky factor of every wavenumber's matrix in band storage and one forward
and backward substitution per source, as the reference's direct solve
(core/src/bert/dcfemmodelling.cpp:2199-2210).

GPU: every 2-D golden case against the reference's fixtures (potentials and
apparent resistivities <= 1e-6, Jacobian <= 1e-5; observed at the level of
the fixtures' own direct solve), the 41-electrode 2.5-D configuration
against the oracle, a reverse-Cuthill-McKee ordering (the mesh renumbered at
random), a batch of such problems side by side, and the refusal of a matrix
whose bandwidth exceeds 256 (a 3-D box)."""
import os

import numpy as np
import pytest

from oracle import ert_oracle as O
from pygimli_gb300.data import DataContainerERT
from pygimli_gb300.mesh import Mesh

pytestmark = pytest.mark.gpu

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


def load_case(golden_dir, name):
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"], z["boundaries"],
                z["boundary_markers"], z["boundary_cells"])
    if int(z["p2"]) == 1:
        mesh = mesh.createP2()
    elif int(z["p2"]) == 2:
        mesh = mesh.createH2()
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", z["kfac"])
    return z, mesh, data


def band_fop(mesh, data, **kw):
    from pygimli_gb300 import ERTModelling
    f = ERTModelling(precision="fp64", precond="band", **kw)
    f.setData(data)
    f.setMesh(mesh, ignoreRegionManager=True)
    return f


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("name", ["ert2d_small", "ert2d_pd_wa", "ert2d_p2_small", "ert2d_h2_small"])
def test_golden_2d(torch, golden_dir, name):
    z, mesh, data = load_case(golden_dir, name)
    fop = band_fop(mesh, data)
    rhoa = fop.response(z["rho"])
    e_rhoa = float(np.max(np.abs(rhoa - z["rhoa"]) / z["rhoa"]))
    e_pot = rel(fop.subPotentials(), z["subpot"])
    J = fop.createJacobian(z["rho"]).cpu().numpy()
    e_J = float(np.linalg.norm(J - z["J"]) / np.linalg.norm(z["J"]))
    print(f"{name} band: rhoa {e_rhoa:.2e} potentials {e_pot:.2e} J {e_J:.2e} iterations {fop.stats()['iterations']}")
    assert e_rhoa <= TOL_POT and e_pot <= TOL_POT and e_J <= TOL_J
    assert fop.stats()["iterations"] == 0


def test_c1_vs_oracle(torch):
    """41 electrodes, 741 dipole-dipole data, 17 wavenumbers, against the
    oracle's SuperLU solve."""
    from pygimli_gb300 import synthetic
    from pygimli_gb300.kwave import init_kwave_list
    mesh, data, rho = synthetic.line_2d()[:3]
    k, w = init_kwave_list(2, data.sensorPositions())
    P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], k, w)
    ro, uo = P.response(rho)
    fop = band_fop(mesh, data)
    r = fop.response(rho)
    e = float(np.max(np.abs(r - ro) / ro))
    e_u = rel(fop.subPotentials(), uo)
    print(f"line_2d band vs oracle: rhoa {e:.2e} potentials {e_u:.2e}")
    assert e <= 1e-9 and e_u <= 1e-9


def test_rcm_ordering(torch, golden_dir):
    """The mesh's nodes renumbered at random (bandwidth ~n): the reverse
    Cuthill-McKee order brings it back within the band limit; the response
    equals the one on the original numbering."""
    z, mesh, data = load_case(golden_dir, "ert2d_small")
    n = mesh.nodeCount()
    p = np.random.default_rng(5).permutation(n)  # new index of old node i: p[i]
    inv = np.argsort(p)
    m2 = Mesh(2, mesh.nodes[inv], p[mesh.cells], mesh.cell_markers, mesh.node_markers[inv], p[mesh.boundaries],
              mesh.boundary_markers, mesh.boundary_cells)
    r1 = band_fop(mesh, data).response(z["rho"])
    r2 = band_fop(m2, data).response(z["rho"])
    assert float(np.max(np.abs(r2 - r1) / r1)) <= 1e-9


def test_batch_of_band_problems(torch):
    from pygimli_gb300 import synthetic
    from pygimli_gb300.batch import BatchedERTModelling
    probs = synthetic.batch_2d(5, seed=17, nodes=(1500, 9000), electrodes=(12, 30))
    singles = [band_fop(m, d) for m, d, _ in probs]
    ref = [f.response(r) for f, (_, _, r) in zip(singles, probs)]
    batch = BatchedERTModelling([band_fop(m, d) for m, d, _ in probs])
    out = batch.response([r for _, _, r in probs])
    for i, (o, r) in enumerate(zip(out, ref)):
        assert float(np.max(np.abs(o - r) / r)) <= 1e-12, i


def test_refuses_wide_band(torch, golden_dir):
    from pygimli_gb300._native import BAD_INPUT, ErtgbError
    from pygimli_gb300 import synthetic
    mesh, data, rho = synthetic.box_3d()[:3]
    fop = band_fop(mesh, data)
    with pytest.raises(ErtgbError) as e:
        fop.response(rho)
    assert e.value.code == BAD_INPUT and "bandwidth" in str(e.value)
