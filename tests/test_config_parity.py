"""GPU parity on the benchmarked 3-D configurations against the FP64 oracle.

box_3d (96 electrodes on 12 x 8, 5336 data, 87,696 nodes, 485,640
tetrahedra) and box_3d_large (256 electrodes on 16 x 16, 7392 data, 144,648
nodes, 806,760 tetrahedra), each with its seeded benchmark model.  The
oracle (oracle/ert_oracle.py, the numpy restatement pinned to the
reference's own outputs) assembles the same system, factors it once with
SuperLU and solves the singularity-removal right-hand sides of a seeded
sample of electrodes: one x line and one y line of the grid.  Every datum
whose four electrodes lie in the sample (or are at infinity) is compared for
every solver form, including the learned preconditioner of the headline:

* potentials of the sampled sources: max |u - u_o| / max |u_o| <= 1e-6,
* apparent resistivities: max |rhoa - rhoa_o| / rhoa_o <= 1e-6,
* Jacobian rows (FP64 J for the FP64 form, FP32 J otherwise, the form
  each is timed with): ||J - J_o||_F / ||J_o||_F <= 1e-5.

The errors are printed for every form (``pytest -s``)."""
import os

import numpy as np
import pytest
import scipy.sparse.linalg as spla

from oracle import ert_oracle as O

pytestmark = pytest.mark.gpu

TOL_POT = 1e-6
TOL_J = 1e-5
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FORMS = {"fp64": dict(precision="fp64", precond="jacobi"),
         "mixed": dict(precision="mixed", precond="jacobi"),
         "mixed-fsai": dict(precision="mixed", precond="fsai"),
         "learned": dict(precision="mixed", precond="learned"),
         "fp64-ic0": dict(precision="fp64", precond="ic0")}


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    from pygimli_gb300 import build
    build.build()
    return t


def _sample(nx, ny, x_line, y_line):
    """Electrodes of grid row y = y_line and grid column x = x_line (index x * ny + y)."""
    return sorted({x * ny + y_line for x in range(nx)} | {x_line * ny + y for y in range(ny)})


def _jacobian_rows(P, u, model, rows, block=8):
    """Oracle Jacobian rows of a one-wavenumber (k = 0) problem from the
    potentials u[0, e] of the electrodes the rows use:
    J[d, c] = (u_a - u_b)_c^T K_c (u_m - u_n)_c * w * kfac_d / model_c^2."""
    cells = P.mesh.cells
    U = np.vstack([u[0], np.zeros((1, u.shape[2]))])  # index -1: zero potential
    ab = np.where(P.abmn[rows] < 0, len(U) - 1, P.abmn[rows])
    out = np.empty((len(rows), len(cells)))
    for i in range(0, len(rows), block):
        q = ab[i:i + block]
        dab = U[q[:, 0]][:, cells] - U[q[:, 1]][:, cells]  # rows x C x nv
        dmn = U[q[:, 2]][:, cells] - U[q[:, 3]][:, cells]
        out[i:i + block] = np.einsum("cij,rcj,rci->rc", P.K, dab, dmn) * P.w[0]
    return out * P.kfac[rows][:, None] / (np.asarray(model) ** 2)[None, :]


class ConfigOracle:
    def __init__(self, name):
        from pygimli_gb300 import synthetic
        from pygimli_gb300.kwave import init_kwave_list
        self.name = name
        if name == "box_3d":
            self.mesh, self.data, self.rho = synthetic.box_3d()
            sample = _sample(12, 8, 5, 3)
        else:
            self.mesh, self.data, self.rho = synthetic.box_3d_large()
            sample = _sample(16, 16, 8, 7)
        k, w = init_kwave_list(3, self.data.sensorPositions())
        P = O.Problem(self.mesh, self.data.sensorPositions(), self.data.abmn(), self.data["k"], k, w)
        ab = self.data.abmn()
        inside = np.isin(ab, sample) | (ab == -1)
        self.rows = np.nonzero(inside.all(axis=1))[0]
        self.sample = np.array(sample)
        # oracle potentials of the sampled sources (singularity removal, one wavenumber)
        rs = P.source_rho(self.rho)
        S = P.csr(P.assemble(self.rho, 0))
        S1 = P.csr(P.assemble(np.ones_like(self.rho), 0))
        lu = spla.splu(S.tocsc(), permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0)
        u = np.zeros((1, P.nE, P.n))
        for e in self.sample:
            prim = P.up[0, e] * rs[e]
            u[0, e] = lu.solve(S1 @ prim / rs[e] - S @ prim) + prim
        self.u = u
        self.rhoa = P.response_from_u(u)[self.rows]
        self.J = _jacobian_rows(P, u, self.rho, self.rows)


_ORACLES = {}


def oracle_for(name):
    if name not in _ORACLES:
        _ORACLES[name] = ConfigOracle(name)
    return _ORACLES[name]


def _weights(name):
    return os.path.join(ROOT, "pygimli_gb300", "weights", "box_3d.npz")


@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("name", ["box_3d", "box_3d_large"])
def test_benchmark_config_vs_oracle(torch, name, form):
    from pygimli_gb300 import ERTModelling
    o = oracle_for(name)
    f = FORMS[form]
    fop = ERTModelling(precision=f["precision"], precond=f["precond"],
                       weights=_weights(name) if f["precond"] == "learned" else None)
    fop.setData(o.data)
    fop.setMesh(o.mesh, ignoreRegionManager=True)
    rhoa = fop.response(o.rho)
    st = fop.stats()
    u = fop.subPotentials()
    e_pot = float(np.max(np.abs(u[0, o.sample] - o.u[0, o.sample])) / np.max(np.abs(o.u[0, o.sample])))
    e_rhoa = float(np.max(np.abs(rhoa[o.rows] - o.rhoa) / o.rhoa))
    jdt = "float64" if f["precision"] == "fp64" else "float32"
    J = fop.createJacobian(o.rho, dtype=jdt)
    Jr = J[torch.as_tensor(o.rows, device=J.device)].cpu().numpy().astype(np.float64)
    del J
    e_J = float(np.linalg.norm(Jr - o.J) / np.linalg.norm(o.J))
    print(f"{name} {form}: {len(o.sample)} sources, {len(o.rows)} data; potentials {e_pot:.2e} rhoa {e_rhoa:.2e} "
          f"J({jdt}) {e_J:.2e}; PCG iterations {st['iterations']}, FP64-finished columns {st['stalled_columns']}")
    assert e_pot <= TOL_POT and e_rhoa <= TOL_POT and e_J <= TOL_J
