"""Generate the fixture of the regularised CGLS of a Gauss-Newton step from
the reference's own C++ (solveCGLSCDWWhtrans, core/src/solver.cpp:27-212,
in oracle/_ref/libgimli_ref.so, built by ``make -C oracle``) through
oracle/ref_driver.py:

    python tests/golden/make_cgls_golden.py

Fixture cgls_small.npz: a seeded dense Jacobian (40 x 30), a chain of
first-order constraints (29 rows), data and constraint weights, model and
data transformation derivatives, lambda 3 and a roughness vector; the
reference's solution after 5 iterations (x5; the system's condition is
1.4e7, so later iterates carry amplified summation-order rounding) and
converged (max 500 iterations, tolerance 1e-28 on ||r||^2: xconv).
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_driver  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def main():
    rng = np.random.default_rng(0)
    D, P = 40, 30
    J = rng.normal(size=(D, P))
    R = P - 1
    rp = np.arange(0, 2 * R + 1, 2, dtype=np.int32)
    ci = np.empty(2 * R, np.int32)
    ci[0::2], ci[1::2] = np.arange(R), np.arange(1, P)
    cv = np.tile([1.0, -1.0], R)
    v = dict(dW=rng.uniform(5, 20, D), b=rng.normal(size=D), wc=rng.uniform(0.5, 1.5, R), wm=np.ones(P),
             tm=rng.uniform(0.01, 0.1, P), td=rng.uniform(0.01, 0.1, D), rough=rng.normal(size=R) * 0.1)
    lam = 3.0
    args = (J, (rp, ci, cv, P), v["dW"], v["b"], np.zeros(P), v["wc"], v["wm"], v["tm"], v["td"], lam, v["rough"])
    x5 = ref_driver.cgls(*args, max_iter=5, tol=-1.0)
    xconv = ref_driver.cgls(*args, max_iter=500, tol=1e-28)
    np.savez_compressed(os.path.join(OUT, "cgls_small.npz"), J=J, rp=rp, ci=ci, cv=cv, lam=lam, x5=x5,
                        xconv=xconv, **v)
    print("cgls_small", J.shape, "|x5|", np.linalg.norm(x5), "|xconv|", np.linalg.norm(xconv))


if __name__ == "__main__":
    main()
