"""Learned preconditioner: the FP64 oracle against finite differences (CPU),
the CUDA network, loss and gradients against the oracle (GPU), and what the
trained network gains over the solver without it (GPU).

Tolerances: features 1e-5 relative (FP32 storage of FP64 arithmetic); the
network's factor G 3e-2 and the gradient blocks 6e-2 in the relative
Frobenius norm, from the BF16 storage of activations and BF16 tensor-core
operands (2^-9 relative rounding per stored value, compounded over four
residual layers); the loss 5e-3 absolute (about 0.3% of its value, the
effect of the BF16-rounded factor on log-traces and log-diagonals)."""
import os

import numpy as np
import pytest

from oracle import ert_oracle as O
from oracle import learned_oracle as LO
from pygimli_gb300.data import DataContainerERT, createData, geometricFactors, grid_line_scheme
from pygimli_gb300.kwave import init_kwave_list
from pygimli_gb300.mesh import create_box_mesh_3d, create_para_mesh_2d

TOL_FEAT = 1e-5
TOL_G = 3e-2
TOL_GRAD = 6e-2
TOL_LOSS = 5e-3


def _small_2d(n_el=5, dx=1.0, depth=2.0):
    xs = np.arange(float(n_el))
    mesh = create_para_mesh_2d(xs, para_dx=dx, para_depth=depth)
    data = createData(xs, "dd")
    data.set("k", geometricFactors(data, 2))
    return mesh, data


def test_oracle_gradient_matches_finite_differences():
    mesh, data = _small_2d()
    k, w = init_kwave_list(2, data.sensorPositions())
    P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], k, w)
    rng = np.random.default_rng(0)
    A = P.assemble(np.exp(rng.uniform(0, 3, mesh.cellCount())), 2)
    g = LO.Graph(P.rowptr, P.cols)
    theta = LO.init_params(1, decoder_scale=0.05)
    feats = LO.features(g, A)
    L, grad, _ = LO.loss_and_grad(theta, g, A, feats)
    off = 0
    for name, shape in LO.param_layout():
        n = int(np.prod(shape))
        i = off + int(rng.integers(n))
        h = 1e-6
        t1, t2 = theta.copy(), theta.copy()
        t1[i] += h
        t2[i] -= h
        fd = (LO.loss_and_grad(t1, g, A, feats)[0] - LO.loss_and_grad(t2, g, A, feats)[0]) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-4 * (abs(grad[i]) + 1e-3 * np.abs(grad).max()), name
        off += n


def test_oracle_fsai_minimises_kaporin():
    """FSAI is the minimiser of the training loss on A's lower pattern."""
    mesh, data = _small_2d()
    k, w = init_kwave_list(2, data.sensorPositions())
    P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], k, w)
    A = P.assemble(np.full(mesh.cellCount(), 30.0), 1)
    g = LO.Graph(P.rowptr, P.cols)
    GF = LO.fsai(g, A)
    K0, dG = LO.kaporin(g, A, GF)
    assert np.max(np.abs(dG)) < 1e-10 * np.max(np.abs(GF))
    rng = np.random.default_rng(3)
    for _ in range(3):
        assert LO.kaporin(g, A, GF * (1 + 0.05 * rng.normal(size=GF.size)))[0] > K0


# ------------------------------------------------------------------ GPU
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
    fop = ERTModelling(**kw)
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    return fop


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.gpu
def test_features_forward_loss_gradient_vs_oracle(torch):
    mesh, data = _small_2d(7, 0.5, 3.0)
    fop = _fop(mesh, data)
    rng = np.random.default_rng(1)
    rho = np.exp(rng.normal(np.log(100.0), 1.0, mesh.cellCount()))
    fop.assemble(rho)
    rp, ci = fop.pattern()
    g = LO.Graph(rp, ci)
    theta64 = LO.init_params(2, decoder_scale=0.05)
    theta = torch.tensor(theta64.astype(np.float32), device="cuda")
    theta_o = theta.cpu().numpy().astype(np.float64)
    x_d, f_d = fop.lpFeatures()
    G_d = fop.lpForward(theta).cpu().numpy()
    grad = torch.zeros_like(theta)
    loss_d = fop.lpLossGrad(theta, grad)
    grad_d = grad.cpu().numpy().astype(np.float64)
    nK = len(fop.kValues())
    losses, grads = [], []
    for ki in range(nK):
        A = fop.matrix(ki, 0)
        x, f = LO.features(g, A)
        assert _rel(x_d[ki].cpu().numpy(), x) <= TOL_FEAT and _rel(f_d[ki].cpu().numpy(), f) <= TOL_FEAT
        L, gr, G = LO.loss_and_grad(theta_o, g, A, (x, f))
        eG = _rel(G_d[ki], G)
        print(f"k {ki}: G rel {eG:.2e}")
        assert eG <= TOL_G, ki
        losses.append(L)
        grads.append(gr)
    loss_o = float(np.mean(losses))
    grad_o = np.mean(grads, axis=0)
    print(f"loss gpu {loss_d:.6f} oracle {loss_o:.6f}")
    assert abs(loss_d - loss_o) <= TOL_LOSS
    off = 0
    for name, shape in LO.param_layout():
        n = int(np.prod(shape))
        e = _rel(grad_d[off:off + n], grad_o[off:off + n])
        print(f"grad {name}: rel {e:.2e}")
        assert e <= TOL_GRAD, name
        off += n


def _box_case(seed_models, nx=6, ny=4):
    e = np.array([(x, y) for x in np.arange(nx) * 4.0 for y in np.arange(ny) * 4.0])
    mesh = create_box_mesh_3d(e, h=2.0, para_margin=(2, 2), para_depth=8.0, outer=100.0, growth=1.8,
                              depth_growth=1.4)
    data = DataContainerERT(np.column_stack([e, np.zeros(len(e))]), grid_line_scheme((nx, ny), "dd"))
    data.set("k", geometricFactors(data, 3))
    models = []
    c = mesh.cellCenters()
    for s in seed_models:
        rng = np.random.default_rng(s)
        rho = np.exp(rng.normal(np.log(100.0), 1.0, mesh.cellCount()))
        for _ in range(2):
            ctr = rng.uniform([0, 0, -8], [4 * nx, 4 * ny, -1])
            ax = rng.uniform(2.0, 6.0, 3)
            rho[np.sum(((c - ctr) / ax) ** 2, axis=1) < 1.0] = 10 ** rng.uniform(0.5, 4.5)
        models.append(rho)
    return mesh, data, models


@pytest.mark.gpu
def test_training_gains_over_jacobi(torch):
    """Trained on 8 models, evaluated on 2 held-out ones: fewer PCG iterations
    than the mixed-precision solver without the network (Jacobi, which is
    also the untrained network), same converged answer."""
    from pygimli_gb300.learned import LearnedPreconditioner
    mesh, data, models = _box_case(range(10))
    train, held = models[:8], models[8:]
    fop = _fop(mesh, data, precision="mixed")
    lp = LearnedPreconditioner(seed=0)
    k0 = np.mean([lp.loss(fop, m) for m in held])
    hist = lp.train(fop, train, steps=240, lr=2e-3)
    k1 = np.mean([lp.loss(fop, m) for m in held])
    its = {}
    rhoa = {}
    for name in ("jacobi", "learned", "fsai"):
        fop.setPreconditioner(name, lp if name == "learned" else None)
        its[name] = 0
        for m in held:
            rhoa[(name, id(m))] = fop.response(m)
            its[name] += fop.stats()["iterations"]
    print(f"held-out Kaporin {k0:.4f} -> {k1:.4f}; iterations {its}; first/last train loss "
          f"{hist[0][1]:.4f}/{hist[-1][1]:.4f}")
    for m in held:
        r0, r1 = rhoa[("jacobi", id(m))], rhoa[("learned", id(m))]
        assert np.max(np.abs(r1 - r0) / r0) <= 1e-6
    assert k1 < k0
    assert its["learned"] <= 0.85 * its["jacobi"]
