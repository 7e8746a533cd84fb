"""Test infrastructure only: FP64 numpy restatement of pyGIMLi's regularised
CGLS (solveCGLSCDWWhtrans, core/src/solver.cpp:27-212), the checker of the
GPU ``ertgb_cgls``.  Same operations in the same order, including the
rounding of C (p wm) to 1e-10.  Pinned to the reference's own
solveCGLSCDWWhtrans run through oracle/_ref (tests/golden/cgls_small.npz,
tests/golden/make_cgls_golden.py; tests/test_inversion.py)."""
from __future__ import annotations

import numpy as np


def _csr_mul(C, x):
    rp, ci, cv, _ = C
    out = np.zeros(len(rp) - 1)
    np.add.at(out, np.repeat(np.arange(len(rp) - 1), np.diff(rp)), cv * x[ci])
    return out


def _csr_tmul(C, y):
    rp, ci, cv, P = C
    out = np.zeros(P)
    np.add.at(out, ci, cv * y[np.repeat(np.arange(len(rp) - 1), np.diff(rp))])
    return out


def cgls(J, C, dW, b, x, wc, wm, tm, td, lam, rough, max_iter=200, tol=-1.0):
    x = np.array(x, np.float64)
    cdx = _csr_tmul(C, wc * rough) * wm * lam
    z = (b - (J @ (x / tm)) * td) * dW
    p = (J.T @ (z * dW * td)) / tm - _csr_tmul(C, wc * wc * _csr_mul(C, wm * x)) * wm * lam - cdx
    r = (J.T @ (b * dW * dW * td)) / tm - cdx
    acc = tol if tol >= 0 else max(1e-12, 1e-8 * float(r @ r))
    r = p.copy()
    nr2 = float(r @ r)
    count = 0
    while count < max_iter and nr2 > acc:
        count += 1
        q = (J @ (p / tm)) * (dW * td)
        cp = np.rint(_csr_mul(C, p * wm) / 1e-10) * 1e-10
        wcp = wc * cp
        aq = float(q @ q) + lam * float(wcp @ wcp)
        alpha = nr2 / aq
        x += alpha * p
        z -= alpha * q
        r = (J.T @ (z * dW * td)) / tm - _csr_tmul(C, wc * wc * _csr_mul(C, wm * x)) * wm * lam - cdx
        old = nr2
        nr2 = float(r @ r)
        p = r + (nr2 / old) * p
    return x, count
