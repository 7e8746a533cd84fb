"""The dipole current pattern (DCMultiElectrodeModelling::
setDipoleCurrentPattern + calculate(DataContainerERT &), core/src/bert/
dcfemmodelling.cpp:1488-1513, 1558-1618): one current pattern per distinct
(a, b) pair of the data, the voltages u = pot_m - pot_n of the datum's
pattern for a unit current, no reference electrode (a pole datum of a closed
domain drains at the calibration nodes).  Fixtures from the reference's own
C++ (tests/golden/make_dipole_golden.py).

Here every (a, b) pattern is the difference of the pure poles a and b,
which is exact: one system matrix per wavenumber for all sources, a
right-hand side linear in the source, and a singularity-removal potential
that does not depend on the source resistivity at the free nodes.

CPU: the oracle (pure poles, dipole=True) against the reference's dipole
solves, voltages <= 1e-9 of the largest (complete-electrode-model and
bypass electrodes too; the bypass resistors' conditioning: 1e-8); the closed-domain
singularity-removal primaries, which the reference takes per (a, b) pattern,
equal the oracle's pole differences (<= 1e-8).  GPU: ``calculate`` in the
dipole mode against the same fixtures (<= 1e-6), ``calculate`` of pole
patterns with electrodes inside cells against the oracle, and the refusals
(``response``/``createJacobian`` in the dipole mode, a pattern the data do
not hold, a measuring electrode on a fixed-potential node with singularity
removal)."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))

import cem_oracle as CO  # noqa: E402
from oracle import ert_oracle as O  # noqa: E402
from pygimli_gb300.data import DataContainerERT  # noqa: E402
from pygimli_gb300.mesh import Mesh  # noqa: E402

CASES = ["ert3d_dipole_sr_small", "ert3d_dipole_tp_small", "ert3d_dipole_closed_tp_small",
         "ert3d_dipole_closed_sr_small", "ert2d_dipole_sr_small", "ert2d_dipole_tp_small"]
CEM_CASES = ["ert2d_dipole_cem_small", "ert3d_dipole_cem_small", "ert2d_dipole_bypass_small"]
TOL_ORACLE = 1e-9
TOL_GPU = 1e-6


def load(golden_dir, name):
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"], z["boundaries"],
                z["boundary_markers"], z["boundary_cells"], check=False)
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", np.ones(data.size()))  # voltages only: the factors do not enter
    return z, mesh, data


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def oracle_problem(z, mesh, data):
    args = (mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"])
    if int(z["sr"]):
        prim = None
        if z["primary"].size:
            prim = O.numerical_primary(*args, dipole=True)
        return O.Problem(*args, primary=prim, dipole=True), prim
    return CO.TotalPotentialProblem(*args, dipole=True), None


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(golden_dir, name):
    z, mesh, data = load(golden_dir, name)
    P, prim = oracle_problem(z, mesh, data)
    assert P.sink is None  # no reference electrode with the dipole pattern
    if prim is not None:
        # the reference's primaries of the (a, b) patterns = differences of the poles
        pats = z["patterns"]
        p0 = prim[0]
        pole = lambda e: p0[e] if e >= 0 else np.zeros(p0.shape[1])  # noqa: E731
        dip = np.array([pole(a) - pole(b) for a, b in pats])
        assert rel(dip, z["primary"]) <= 1e-8
    u = P.calculate(z["rho"])
    assert rel(u, z["u"]) <= TOL_ORACLE


@pytest.mark.parametrize("name", CEM_CASES)
def test_oracle_cem_matches_reference(golden_dir, name):
    """The dipole pattern with complete-electrode-model and bypass
    electrodes (total potential, the reference's calculate with its CEM
    potentials): the differences of the oracle's pure poles."""
    z, mesh, data = load(golden_dir, name)
    zc = z["contact_impedance"]
    P = CO.TotalPotentialProblem(mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"],
                                 contact_impedance=zc if len(zc) else None, dipole=True)
    assert rel(P.calculate(z["rho"]), z["u"]) <= (1e-8 if "bypass" in name else TOL_ORACLE)


def test_pattern_count_and_order(golden_dir):
    """The reference solved one pattern per distinct (a, b) pair, in the
    order of its pattern index (a + 1)(nSensors + 1) + b + 1."""
    for name in CASES + CEM_CASES:
        z, _, data = load(golden_dir, name)
        ab = data.abmn()[:, :2].astype(np.int64)
        assert int(z["n_patterns"]) == len({tuple(p) for p in ab.tolist()})
        idx = (z["patterns"][:, 0] + 1) * (data.sensorCount() + 1) + z["patterns"][:, 1] + 1
        assert np.all(np.diff(idx) > 0)


def test_host_boundary_setup():
    """Host and oracle agree: no reference with the dipole pattern, the
    calibration nodes stay."""
    from pygimli_gb300.ert import boundary_setup
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    z, mesh, data = load(here, "ert3d_dipole_closed_tp_small")
    nE = data.sensorCount()
    for dipole in (False, True):
        h = boundary_setup(mesh, nE, dipole)
        o = O.BoundarySetup(mesh, nE, dipole)
        assert (h.ref_node, h.ref_elec) == (o.ref_node, o.ref_elec)
        assert np.array_equal(np.sort(h.calib), np.sort(o.calib))
        assert len(h.calib) == 1 and mesh.node_markers[h.calib[0]] == -1000
    assert boundary_setup(mesh, nE, False).ref_node >= 0
    assert boundary_setup(mesh, nE, True).ref_node == -1


def _gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _fop(z, mesh, data, **kw):
    from pygimli_gb300 import ERTModelling
    fop = ERTModelling(sr=bool(int(z["sr"])), **kw)
    fop.setkValues(z["k"])
    fop.setWeights(z["w"])
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    return fop


@pytest.mark.gpu
@pytest.mark.parametrize("form", ["fp64", "mixed-fsai"])
@pytest.mark.parametrize("name", CASES)
def test_gpu_calculate_matches_reference(golden_dir, name, form):
    _gpu()
    z, mesh, data = load(golden_dir, name)
    kw = dict(precision="fp64") if form == "fp64" else dict(precision="mixed", precond="fsai")
    fop = _fop(z, mesh, data, **kw)
    fop.setDipoleCurrentPattern(True)
    assert fop.dipoleCurrentPattern()
    fop.mapERTModel(z["rho"])
    u = fop.calculate()
    e = rel(u, z["u"])
    print(f"{name} {form}: dipole voltages {e:.2e}")
    assert e <= TOL_GPU
    assert np.array_equal(data["u"], u)


@pytest.mark.gpu
def test_gpu_pole_and_dipole_modes():
    """With mixed boundaries and no reference the pole patterns' voltages are
    the dipole ones; in a closed domain the pole mode returns the current
    through the reference node (-999) and only a pole datum (b = -1) differs;
    switching back restores response and the Jacobian."""
    _gpu()
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    z, mesh, data = load(here, "ert3d_dipole_sr_small")
    fop = _fop(z, mesh, data, precision="fp64")
    rhoa = fop.response(z["rho"])
    u_pole = fop.calculate()
    assert rel(u_pole, z["u"]) <= TOL_GPU
    fop.setDipoleCurrentPattern(True)
    with pytest.raises(NotImplementedError):
        fop.response(z["rho"])
    with pytest.raises(NotImplementedError):
        fop.createJacobian(z["rho"])
    fop.setDipoleCurrentPattern(False)
    assert rel(fop.response(z["rho"]), rhoa) <= 1e-12
    assert fop.createJacobian(z["rho"]).shape == (data.size(), mesh.cellCount())
    z, mesh, data = load(here, "ert3d_dipole_closed_tp_small")
    fop = _fop(z, mesh, data, precision="fp64")
    fop.mapERTModel(z["rho"])
    u_pole = fop.calculate()
    pole_datum = np.flatnonzero(data.abmn()[:, 1] == -1)
    other = np.setdiff1d(np.arange(data.size()), pole_datum)
    assert rel(u_pole[other], z["u"][other]) <= TOL_GPU
    assert np.all(np.abs(u_pole[pole_datum] - z["u"][pole_datum]) > 1e-3 * np.abs(z["u"]).max())


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ert3d_entity_small", "ert2d_entity_tp_small"])
def test_gpu_calculate_entity_electrodes(golden_dir, name):
    """Voltages of electrodes inside cells: the collect interpolates with the
    cell's shape functions (oracle, pole patterns)."""
    _gpu()
    z = np.load(os.path.join(golden_dir, name + ".npz"))
    mesh = Mesh(int(z["dim"]), z["nodes"], z["cells"], z["cell_markers"], z["node_markers"], z["boundaries"],
                z["boundary_markers"], z["boundary_cells"], check=False)
    data = DataContainerERT(z["sensors"], z["abmn"])
    data.set("k", z["kfac"])
    args = (mesh, data.sensorPositions(), data.abmn(), data["k"], z["k"], z["w"])
    P = O.Problem(*args) if int(z["sr"]) else CO.TotalPotentialProblem(*args)
    u_o = P.calculate(z["rho"])
    fop = _fop(z, mesh, data, precision="fp64")
    fop.response(z["rho"])
    u = fop.calculate()
    e = rel(u, u_o)
    print(f"{name}: voltages {e:.2e}")
    assert e <= TOL_GPU


@pytest.mark.gpu
def test_gpu_dipole_refusals(golden_dir):
    _gpu()
    z, mesh, data = load(golden_dir, "ert3d_dipole_closed_sr_small")
    fop = _fop(z, mesh, data, precision="fp64")
    fop.setDipoleCurrentPattern(True)
    with pytest.raises(RuntimeError):
        fop.calculate()  # no model mapped yet
    fop.mapERTModel(z["rho"])
    other = DataContainerERT(z["sensors"], np.array([[3, 5, 0, 1]], np.int32))
    with pytest.raises(ValueError, match="not among"):
        fop.calculate(other)
    # a measuring electrode inside a cell at a homogeneous Dirichlet node
    zd = np.load(os.path.join(golden_dir, "ert3d_dirichlet_sr_small.npz"))
    md = Mesh(3, zd["nodes"], zd["cells"], zd["cell_markers"], zd["node_markers"], zd["boundaries"],
              zd["boundary_markers"], zd["boundary_cells"], check=False)
    dn = int(md.boundaries[md.boundary_markers == -3][0, 0])
    cell = int(np.flatnonzero(np.any(md.cells == dn, axis=1))[0])
    sensors = np.vstack([zd["sensors"], md.nodes[md.cells[cell]].mean(axis=0)])
    ab = np.vstack([zd["abmn"], [[0, 1, 2, len(sensors) - 1]]]).astype(np.int32)
    d2 = DataContainerERT(sensors, ab)
    d2.set("k", np.ones(d2.size()))
    fop = _fop(zd, md, d2, precision="fp64")
    fop.setDipoleCurrentPattern(True)
    fop.mapERTModel(zd["rho"])
    with pytest.raises(NotImplementedError, match="fixed-potential"):
        fop.calculate()
    fop.setDipoleCurrentPattern(False)  # pole patterns: the reference's own values there
    assert np.all(np.isfinite(fop.calculate()))
