"""Batched solve of independent problems (pygimli_gb300.batch): every
problem's apparent resistivities and Jacobian equal those of its own FP64
solve (potentials / rhoa <= 1e-6, Jacobian <= 1e-5 relative), one small
problem is checked against the oracle, and the autotuner's choice is one of
its timed candidates and is cached for an identical batch.  A batch of FP64
operators (their solves side by side) equals the single FP64 solves."""
import numpy as np
import pytest

from oracle import ert_oracle as O

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


def _fop(mesh, data, **kw):
    from pygimli_gb300 import ERTModelling
    f = ERTModelling(**kw)
    f.setData(data)
    f.setMesh(mesh, ignoreRegionManager=True)
    return f


def test_batch_matches_single_solves(torch):
    from pygimli_gb300 import synthetic
    from pygimli_gb300.batch import BatchedERTModelling
    probs = synthetic.batch_2d(6, seed=11, nodes=(1500, 9000), electrodes=(12, 30))
    singles = [_fop(m, d) for m, d, _ in probs]
    ref = [f.response(r) for f, (_, _, r) in zip(singles, probs)]
    Jref = [f.createJacobian(r).cpu().numpy() for f, (_, _, r) in zip(singles, probs)]
    batch = BatchedERTModelling([_fop(m, d, precision="mixed") for m, d, _ in probs])
    out = batch.response([r for _, _, r in probs])
    info = batch.info
    print({k: v for k, v in info.items() if k != "candidates"}, info["candidates"])
    for i, (o, r) in enumerate(zip(out, ref)):
        e = float(np.max(np.abs(o - r) / r))
        assert e <= TOL_POT, (i, e)
    J = batch.createJacobian([r for _, _, r in probs])
    for i, (a, b) in enumerate(zip(J, Jref)):
        assert np.linalg.norm(a.cpu().numpy() - b) <= TOL_J * np.linalg.norm(b), i
    assert (info["rows_per_tile"], info["rhs_width"]) in [(c[0], c[1]) for c in info["candidates"]]
    assert info["spmm_tiles"] > 0 and info["columns"] % 128 == 0
    # smallest problem against the oracle
    i = int(np.argmin([m.nodeCount() for m, _, _ in probs]))
    m, d, r = probs[i]
    f = batch.fops[i]
    P = O.Problem(m, d.sensorPositions(), d.abmn(), d["k"], f.kValues(), f.weights())
    ro, _ = P.response(r)
    assert float(np.max(np.abs(out[i] - ro) / ro)) <= TOL_POT
    # an identical batch reuses the tuned shape
    out2 = batch.response([r * 2.0 for _, _, r in probs])
    assert batch.info["cached"]
    for o2, o in zip(out2, out):
        assert float(np.max(np.abs(o2 - 2.0 * o) / (2.0 * o))) <= TOL_POT


def test_fp64_batch_matches_single_solves(torch):
    """A batch of FP64 operators runs every problem's own FP64 solve side by
    side: the same responses and Jacobians as the single solves (1e-9)."""
    from pygimli_gb300 import synthetic
    from pygimli_gb300.batch import BatchedERTModelling
    probs = synthetic.batch_2d(5, seed=13, nodes=(1500, 9000), electrodes=(12, 30))
    singles = [_fop(m, d) for m, d, _ in probs]
    ref = [f.response(r) for f, (_, _, r) in zip(singles, probs)]
    batch = BatchedERTModelling([_fop(m, d, precision="fp64") for m, d, _ in probs])
    out = batch.response([r for _, _, r in probs])
    for i, (o, r) in enumerate(zip(out, ref)):
        e = float(np.max(np.abs(o - r) / r))
        assert e <= 1e-9, (i, e)
    J = batch.createJacobian([r for _, _, r in probs])
    for i, (f, (_, _, r)) in enumerate(zip(singles, probs)):
        Jr = f.createJacobian(r).cpu().numpy()
        assert np.linalg.norm(J[i].cpu().numpy() - Jr) <= 1e-9 * np.linalg.norm(Jr), i
    assert batch.info["iterations"] > 0 and batch.info["stalled_columns"] == 0


def test_batch_errors(torch):
    from pygimli_gb300 import synthetic
    from pygimli_gb300.batch import BatchedERTModelling
    (m, d, r), = synthetic.batch_2d(1, seed=2, nodes=(1500, 2500), electrodes=(12, 14))
    f = _fop(m, d)
    with pytest.raises(ValueError):
        BatchedERTModelling([f, f])
    b = BatchedERTModelling([f])
    bad = r.copy()
    bad[3] = -1.0
    with pytest.raises(ValueError):
        b.response([bad])
    rr = b.response([r])[0]
    assert np.all(np.isfinite(rr))
