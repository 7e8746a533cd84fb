"""Gauss-Newton step: the oracle CGLS against the normal equations (CPU),
the GPU CGLS against the oracle on the same Jacobian (GPU, 1e-9 relative
for an FP64 Jacobian, 1e-4 for an FP32 one whose products run in FP32, after
15 iterations: the random test system has condition 1.4e7, and CG
amplifies a one-ulp change of J to 2e-13 by iteration 20 and to 3e-4 by
iteration 60, so later iterates are not comparable between any two
summation orders), and a full step that lowers the objective."""
import numpy as np
import pytest

from oracle import inversion_oracle as IO


def _random_problem(seed=0, D=40, P=30):
    rng = np.random.default_rng(seed)
    J = rng.normal(size=(D, P))
    # a chain of first-order constraints
    R = P - 1
    rp = np.arange(0, 2 * R + 1, 2, dtype=np.int32)
    ci = np.empty(2 * R, np.int32)
    ci[0::2], ci[1::2] = np.arange(R), np.arange(1, P)
    cv = np.tile([1.0, -1.0], R)
    C = (rp, ci, cv, P)
    v = dict(dW=rng.uniform(5, 20, D), b=rng.normal(size=D), wc=rng.uniform(0.5, 1.5, R), wm=np.ones(P),
             tm=rng.uniform(0.01, 0.1, P), td=rng.uniform(0.01, 0.1, D), rough=rng.normal(size=R) * 0.1)
    return J, C, v


def test_oracle_cgls_solves_normal_equations():
    J, C, v = _random_problem()
    lam = 3.0
    x, it = IO.cgls(J, C, v["dW"], v["b"], np.zeros(J.shape[1]), v["wc"], v["wm"], v["tm"], v["td"], lam, v["rough"],
                    max_iter=500, tol=1e-28)
    rp, ci, cv, P = C
    Cd = np.zeros((len(rp) - 1, P))
    Cd[np.repeat(np.arange(len(rp) - 1), 2), ci] = cv
    Jt = (v["td"][:, None] * J) / v["tm"][None, :]
    Wd = np.diag(v["dW"] ** 2)
    Cw = v["wc"][:, None] * Cd * v["wm"][None, :]
    A = Jt.T @ Wd @ Jt + lam * Cw.T @ Cw
    rhs = Jt.T @ Wd @ v["b"] - lam * (Cd.T @ (v["wc"] * v["rough"])) * v["wm"]
    xs = np.linalg.solve(A, rhs)
    assert np.linalg.norm(x - xs) <= 1e-8 * np.linalg.norm(xs)


def _golden(golden_dir):
    z = np.load(golden_dir + "/cgls_small.npz")
    C = (z["rp"], z["ci"], z["cv"], z["J"].shape[1])
    args = (z["J"], C, z["dW"], z["b"], np.zeros(z["J"].shape[1]), z["wc"], z["wm"], z["tm"], z["td"], float(z["lam"]),
            z["rough"])
    return z, args


def test_oracle_cgls_matches_reference(golden_dir):
    """The oracle CGLS against the reference's own solveCGLSCDWWhtrans
    (core/src/solver.cpp:27-212, fixture tests/golden/make_cgls_golden.py):
    after 5 iterations and converged."""
    z, args = _golden(golden_dir)
    x5, _ = IO.cgls(*args, max_iter=5)
    assert np.linalg.norm(x5 - z["x5"]) <= 1e-12 * np.linalg.norm(z["x5"])
    xc, _ = IO.cgls(*args, max_iter=500, tol=1e-28)
    assert np.linalg.norm(xc - z["xconv"]) <= 1e-9 * np.linalg.norm(z["xconv"])


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    from pygimli_gb300 import build
    build.build()
    return t


@pytest.mark.gpu
# FP32 Jacobian: the GPU forms the products in FP32 (per-thread partial sums)
# while the oracle uses FP64 arithmetic on the same FP32 values: 1e-4
@pytest.mark.parametrize("dtype,tol", [("float64", 1e-9), ("float32", 1e-4)])
def test_gpu_cgls_matches_oracle(torch, dtype, tol):
    from pygimli_gb300.inversion import cgls
    J, C, v = _random_problem(seed=1, D=300, P=700)
    Jd = torch.tensor(J, dtype=getattr(torch, dtype), device="cuda")
    Jo = Jd.cpu().numpy().astype(np.float64)
    args = (C, v["dW"], v["b"], np.zeros(J.shape[1]), v["wc"], v["wm"], v["tm"], v["td"], 2.0, v["rough"])
    xg, itg = cgls(Jd, *args, max_iter=15)
    xo, ito = IO.cgls(Jo, *args, max_iter=15)
    assert itg == ito
    assert np.linalg.norm(xg - xo) <= tol * np.linalg.norm(xo)


@pytest.mark.gpu
def test_gauss_newton_step_lowers_objective(torch):
    from pygimli_gb300 import ERTModelling
    from pygimli_gb300.data import createData, geometricFactors
    from pygimli_gb300.inversion import GaussNewton
    from pygimli_gb300.mesh import create_para_mesh_2d
    xs = np.arange(21.0)
    mesh = create_para_mesh_2d(xs, para_dx=0.5, para_depth=5.0)
    data = createData(xs, "dd")
    data.set("k", geometricFactors(data, 2))
    rng = np.random.default_rng(4)
    c = mesh.cellCenters()
    true = np.full(mesh.cellCount(), 100.0)
    true[(np.abs(c[:, 0] - 10) < 2.5) & (c[:, 1] > -3) & (c[:, 1] < -1)] = 20.0
    fop = ERTModelling()
    fop.setData(data)
    fop.setMesh(mesh, ignoreRegionManager=True)
    obs = fop.response(true) * (1 + 0.01 * rng.normal(size=data.size()))
    gn = GaussNewton(fop, obs, np.full(data.size(), 0.02), lam=20.0)
    model = np.full(mesh.cellCount(), float(np.median(obs)))
    resp = fop.response(model)
    phi0 = gn.phi(model, resp)
    for _ in range(3):
        model, resp, info = gn.step(model, resp)
        print(info)
        assert 0.0 < info["tau"] <= 1.0 and info["cgls_iterations"] > 0
    assert gn.phi(model, resp) < 0.5 * phi0
    # the anomaly is recovered as conductive
    inside = (np.abs(c[:, 0] - 10) < 2.0) & (c[:, 1] > -2.8) & (c[:, 1] < -1.2)
    assert np.median(model[inside]) < np.median(model[~inside])


@pytest.mark.gpu
def test_gpu_cgls_matches_reference(torch, golden_dir):
    """The GPU CGLS (FP64 Jacobian) against the reference's own
    solveCGLSCDWWhtrans after 5 iterations and converged."""
    from pygimli_gb300.inversion import cgls
    z, args = _golden(golden_dir)
    Jd = torch.tensor(z["J"], dtype=torch.float64, device="cuda")
    x5, _ = cgls(Jd, *args[1:], max_iter=5)
    e5 = float(np.linalg.norm(x5 - z["x5"]) / np.linalg.norm(z["x5"]))
    xc, _ = cgls(Jd, *args[1:], max_iter=500, tol=1e-28)
    ec = float(np.linalg.norm(xc - z["xconv"]) / np.linalg.norm(z["xconv"]))
    print(f"GPU CGLS vs reference: 5 iterations {e5:.2e}, converged {ec:.2e}")
    assert e5 <= 1e-10 and ec <= 1e-8


@pytest.mark.gpu
def test_gauss_newton_with_region_manager(torch):
    """setMesh(mesh) through the region manager (four regions, H2 forward
    mesh): the step takes the region manager's constraint matrix over the
    parameter mesh (RegionManager::fillConstraints, pinned in
    tests/test_regions.py), not rows over the refined forward mesh's faces,
    and lowers the objective."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    from make_regions_golden import region_mesh
    from pygimli_gb300 import ERTModelling
    from pygimli_gb300.data import createData, geometricFactors
    from pygimli_gb300.inversion import GaussNewton
    data = createData(np.arange(9.0), "dd")
    data.set("k", geometricFactors(data, 2))
    fop = ERTModelling()
    fop.setData(data)
    fop.setMesh(region_mesh(2))
    P = fop.parameterCount
    true = np.full(P, 100.0)
    true[: P // 3] = 30.0
    obs = fop.response(true) * (1 + 0.01 * np.random.default_rng(5).normal(size=data.size()))
    gn = GaussNewton(fop, obs, np.full(data.size(), 0.02), lam=20.0)
    rp, ci, cv, Pc = gn.C
    ref = fop.regionManager().constraintMatrix()
    assert Pc == P and np.array_equal(rp, ref[0]) and np.array_equal(ci, ref[1])
    model = np.full(P, float(np.median(obs)))
    resp = fop.response(model)
    phi0 = gn.phi(model, resp)
    model, resp, info = gn.step(model, resp)
    assert gn.phi(model, resp) < phi0
