"""The allocation-free operator entry point (ertgb_csr_spmm_dot_noalloc).

It serves callers that cannot allocate device memory when they call the
library -- a host framework that owns the device memory through its own
pool, or a loop that must not allocate after start-up -- by keeping its
scratch in a fixed array inside the library.  Its results must equal those
of the allocating entry point ertgb_csr_spmm_dot on the same inputs, on
consecutive calls (the fixed scratch keeps the previous call's contents).
This file is collected last so a failure here stops a -x run only after
every other test has run."""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # matrix-value tolerance of the GPU parity tests


@pytest.fixture(scope="module")
def torch():
    t = pytest.importorskip("torch")
    if not t.cuda.is_available():
        pytest.skip("no CUDA device")
    from pygimli_gb300 import build
    build.build()
    return t


def _operator(golden_dir, torch):
    z = np.load(os.path.join(golden_dir, "ert2d_small.npz"))
    rp, ci, vals = z["rowptr"].astype(np.int32), z["colidx"].astype(np.int32), np.ascontiguousarray(z["S"])
    dev = torch.device("cuda")
    return (len(rp) - 1, len(ci), torch.from_numpy(rp).to(dev), torch.from_numpy(ci).to(dev),
            torch.from_numpy(vals).to(dev), vals.shape[0])


def _run(fn, op, X, per_k, torch):
    n, nnz, rp, ci, v, nk = op
    ld = X.shape[1]
    Y = torch.full((n, ld), float("nan"), dtype=torch.float64, device="cuda")
    dots = torch.full((ld,), float("nan"), dtype=torch.float64, device="cuda")
    vp = ctypes.c_void_p
    rc = fn(n, nnz, vp(rp.data_ptr()), vp(ci.data_ptr()), vp(v.data_ptr()), nk, per_k, ld, vp(X.data_ptr()),
            vp(Y.data_ptr()), vp(dots.data_ptr()), vp(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return rc, Y.cpu().numpy(), dots.cpu().numpy()


def test_noalloc_matches_allocating_entry(torch, golden_dir):
    from pygimli_gb300 import _native
    L = _native.load()
    op = _operator(golden_dir, torch)
    rng = np.random.default_rng(5)
    # two calls in a row with different inputs and widths
    for ld, per_k in ((64, 11), (96, 40)):
        X = torch.from_numpy(rng.standard_normal((op[0], ld))).to("cuda")
        rc0, Y0, d0 = _run(L.ertgb_csr_spmm_dot, op, X, per_k, torch)
        rc1, Y1, d1 = _run(L.ertgb_csr_spmm_dot_noalloc, op, X, per_k, torch)
        assert rc0 == 0 and rc1 == 0, L.ertgb_last_error(None)
        assert np.max(np.abs(Y1 - Y0)) <= TOL * np.max(np.abs(Y0))
        assert np.max(np.abs(d1 - d0)) <= TOL * np.max(np.abs(d0))


def test_noalloc_rejects_oversize(torch, golden_dir):
    from pygimli_gb300 import _native
    L = _native.load()
    op = _operator(golden_dir, torch)
    X = torch.zeros((op[0], 1056), dtype=torch.float64, device="cuda")
    rc, _, _ = _run(L.ertgb_csr_spmm_dot_noalloc, op, X, 11, torch)
    assert rc == _native.BAD_INPUT
    assert b"1024" in L.ertgb_last_error(None)
