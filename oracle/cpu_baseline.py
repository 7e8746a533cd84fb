"""Test infrastructure only: timed CPU baseline of the oracle port.

Times the FP64 CPU restatement (oracle/ert_oracle.py; the reference's own
C++ cannot be compiled on a machine without the reference sources) on a
bounded sample of one forward response + Jacobian and extrapolates to the
full workload:

  * per wavenumber: full assembly of S and S1 and one full sparse direct
    factorization (SuperLU, the stand-in for the reference's CHOLMOD);
  * ``n_src`` of the nE current-source solves (+ RHS), scaled by nE/n_src;
  * ``n_rows`` of the D Jacobian rows, scaled by D/n_rows.

Primary potentials are computed once outside the timing, as the reference
caches them (core/src/bert/dcfemmodelling.cpp:1986-2141).  ``threads`` > 1
runs the sampled solves and Jacobian row blocks in a thread pool.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import time

import numpy as np
import scipy.sparse.linalg as spla

from . import ert_oracle as O


def _jacobian_rows(P, u, model, rows):
    cells = P.mesh.cells
    ab = P.abmn[rows]
    out = np.zeros((len(rows), P.mesh.cellCount()))
    for ki, kk in enumerate(P.k):
        S = P.M * (kk * kk) + P.K
        Uc = np.transpose(u[ki][:, cells], (1, 2, 0))
        Uc = np.concatenate([Uc, np.zeros(Uc.shape[:2] + (1,))], axis=2)
        V = np.einsum("cij,cje->cie", S, Uc)
        dab = V[:, :, ab[:, 0]] - V[:, :, ab[:, 1]]
        dmn = Uc[:, :, ab[:, 2]] - Uc[:, :, ab[:, 3]]
        out += P.w[ki] * np.einsum("cid,cid->dc", dab, dmn)
    return out / ((model ** 2)[None, :] / P.kfac[rows][:, None])


class SampledBaseline:
    def __init__(self, mesh, data, k, w):
        self.P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], k, w)

    def step(self, rho, n_src=8, n_rows=64, threads=1, seed=0):
        """Seconds for one full forward + Jacobian, extrapolated from the
        sample; returns (seconds, description)."""
        P = self.P
        nE, D, nK = P.nE, len(P.abmn), len(P.k)
        rng = np.random.default_rng(seed)
        srcs = np.sort(rng.choice(nE, size=min(n_src, nE), replace=False))
        rows = np.sort(rng.choice(D, size=min(n_rows, D), replace=False))
        t0 = time.perf_counter()
        rs = P.source_rho(rho)
        ones = np.ones_like(rho)
        u = np.zeros((nK, nE, P.n))
        t_fixed = 0.0
        t_solve = 0.0
        for ki in range(nK):
            ta = time.perf_counter()
            S = P.csr(P.assemble(rho, ki))
            S1 = P.csr(P.assemble(ones, ki))
            lu = spla.splu(S.tocsc(), permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0)
            tb = time.perf_counter()

            def one(e):
                prim = P.up[ki, e] * rs[e]
                rhs = S1 @ prim / rs[e] - S @ prim
                u[ki, e] = lu.solve(rhs) + prim

            if threads > 1:
                with cf.ThreadPoolExecutor(threads) as ex:
                    list(ex.map(one, srcs))
            else:
                for e in srcs:
                    one(e)
            tc = time.perf_counter()
            t_fixed += tb - ta
            t_solve += tc - tb
        tj0 = time.perf_counter()
        if threads > 1:
            blocks = np.array_split(rows, threads)
            with cf.ThreadPoolExecutor(threads) as ex:
                list(ex.map(lambda r: _jacobian_rows(P, u, rho, r), blocks))
        else:
            _jacobian_rows(P, u, rho, rows)
        t_jac = time.perf_counter() - tj0
        wall = time.perf_counter() - t0
        full = t_fixed + t_solve * (nE / len(srcs)) + t_jac * (D / len(rows))
        desc = (f"{nK} wavenumber(s): full assembly + SuperLU factorization ({t_fixed:.1f} s); "
                f"{len(srcs)}/{nE} source solves ({t_solve:.1f} s); {len(rows)}/{D} Jacobian rows "
                f"({t_jac:.1f} s); sample wall {wall:.1f} s, extrapolated to the full workload")
        return full, desc


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1
