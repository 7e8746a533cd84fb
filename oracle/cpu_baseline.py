"""Test infrastructure only: timed CPU baseline of the oracle port.

Times the FP64 CPU restatement of the reference's forward operator and
Jacobian (oracle/ert_oracle.py; the reference's own C++ is built from the
reference sources, which are not on the machine that runs the benchmark) and
reports the time of one full response + createJacobian, following the cost
structure of the reference's algorithm:

* per wavenumber: assembly of S and S1 and one sparse direct factorization
  (SuperLU, the stand-in for the reference's CHOLMOD), timed in full once
  per run (``factor``) and charged to every step;
* the current-source solves (right-hand side + solve): a seeded sample of
  ``n_src`` sources per step, scaled by nE / n_src (every solve costs the same);
* the Jacobian as the reference computes it (createSensitivityCol_,
  core/src/bert/bertJacobian.cpp:70-119): per cell the products
  V_e = (K_c + k^2 M_c) u_e for every electrode (a fixed cost, over all
  cells every step), then per datum and cell one nv-term dot of two
  differences (the per-datum cost, a seeded sample of ``n_rows`` rows per
  step scaled by D / n_rows).

Cells are processed in blocks so that the per-electrode products of a block
stay small in memory.  Primary potentials are computed once outside the
timing, as the reference caches them (dcfemmodelling.cpp:1986-2141).
``threads`` > 1 runs the sampled solves and the cell blocks in a thread pool.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import time

import numpy as np
import scipy.sparse.linalg as spla

from . import ert_oracle as O

BLOCK = 16384  # cells per block


class SampledBaseline:
    def __init__(self, mesh, data, k, w):
        self.P = O.Problem(mesh, data.sensorPositions(), data.abmn(), data["k"], k, w)
        self.t_factor = None

    def factor(self, rho):
        """Assemble and factor every wavenumber's system (timed)."""
        P = self.P
        t0 = time.perf_counter()
        self.S, self.S1, self.lu = [], [], []
        ones = np.ones_like(rho)
        for ki in range(len(P.k)):
            S = P.csr(P.assemble(rho, ki))
            self.S.append(S)
            self.S1.append(P.csr(P.assemble(ones, ki)))
            self.lu.append(spla.splu(S.tocsc(), permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.0))
        self.t_factor = time.perf_counter() - t0
        return self.t_factor

    def _jacobian(self, u, rows, threads):
        """Per cell block: V = (K + k^2 M) u for every electrode (the fixed
        part, all cells), then the sampled rows' dots.  Returns the wall
        seconds of the two parts (the wall split by the parts' summed
        thread times)."""
        P = self.P
        cells = P.mesh.cells
        ab = P.abmn[rows]
        C = len(cells)

        def one(c0):
            sl = slice(c0, min(c0 + BLOCK, C))
            t_v = t_d = 0.0
            for ki, kk in enumerate(P.k):
                ta = time.perf_counter()
                S = P.M[sl] * (kk * kk) + P.K[sl]
                Uc = np.transpose(u[ki][:, cells[sl]], (1, 2, 0))
                Uc = np.concatenate([Uc, np.zeros(Uc.shape[:2] + (1,))], axis=2)  # index -1 -> 0
                V = np.einsum("cij,cje->cie", S, Uc)
                tb = time.perf_counter()
                dab = V[:, :, ab[:, 0]] - V[:, :, ab[:, 1]]
                dmn = Uc[:, :, ab[:, 2]] - Uc[:, :, ab[:, 3]]
                np.einsum("cid,cid->dc", dab, dmn)
                t_v += tb - ta
                t_d += time.perf_counter() - tb
            return t_v, t_d

        t0 = time.perf_counter()
        starts = range(0, C, BLOCK)
        if threads > 1:
            with cf.ThreadPoolExecutor(threads) as ex:
                parts = list(ex.map(one, starts))
        else:
            parts = [one(c0) for c0 in starts]
        wall = time.perf_counter() - t0
        t_v = sum(p[0] for p in parts)
        t_d = sum(p[1] for p in parts)
        f = t_v / max(t_v + t_d, 1e-30)
        return wall * f, wall * (1.0 - f)

    def step(self, rho, n_src=8, n_rows=64, threads=1, seed=0):
        """Seconds of one full response + Jacobian: the factorization timed
        once per run (in the first step) and charged to every step, the
        Jacobian's per-electrode products over all cells, and samples of the
        solves and of the Jacobian's per-datum dots, scaled.  Returns
        (seconds, description)."""
        P = self.P
        nE, D, nK = P.nE, len(P.abmn), len(P.k)
        rng = np.random.default_rng(seed)
        srcs = np.sort(rng.choice(nE, size=min(n_src, nE), replace=False))
        rows = np.sort(rng.choice(D, size=min(n_rows, D), replace=False))
        if self.t_factor is None:
            self.factor(rho)
        rs = P.source_rho(rho)
        u = np.zeros((nK, nE, P.n))
        t_solve = 0.0
        for ki in range(nK):
            S, S1, lu = self.S[ki], self.S1[ki], self.lu[ki]
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
            t_solve += time.perf_counter() - tb
        t_fixed, t_rows = self._jacobian(u, rows, threads)
        full = self.t_factor + t_solve * (nE / len(srcs)) + t_fixed + t_rows * (D / len(rows))
        desc = (f"{nK} wavenumber(s): assembly + SuperLU factorization {self.t_factor:.1f} s (once per run); "
                f"{len(srcs)}/{nE} source solves {t_solve:.2f} s (scaled); Jacobian per-electrode products "
                f"over all cells {t_fixed:.2f} s + {len(rows)}/{D} rows' dots {t_rows:.2f} s (scaled); "
                f"{threads} thread(s)")
        return full, desc


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:  # pragma: no cover
        return os.cpu_count() or 1
