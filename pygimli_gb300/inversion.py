"""One Gauss-Newton inversion step around the GPU forward operator.

Restates pyGIMLi's classic inversion step (``RInversion::oneStep``,
core/src/inversion.cpp:249-372) for the ERT case: log-transformed data and
model (``TransLog``), first-order smoothness constraints between
neighbouring cells (the region manager's cType 1), data weights 1/error in
the transformed domain, the regularised CGLS model update
(``solveCGLSCDWWhtrans``, core/src/solver.cpp:27-212, here ``ertgb_cgls``
on the GPU with the Jacobian where ``createJacobian`` left it), the update
``m_new = exp(log m + dm)`` and the line search of
``RInversion::linesearch`` (core/src/inversion.h:614-676: 101 step lengths
on the linearised response, a parabolic fit when the best step is below
0.03, a new forward response when the step is below 0.95).

The forward operator is any ``ERTModelling`` whose cell markers are the
parameter indices (one parameter per marker).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native


class TransLog:
    """Logarithmic transformation (pyGIMLi's TransLog with lower bound 0)."""

    @staticmethod
    def trans(v):
        return np.log(v)

    @staticmethod
    def inv(v):
        return np.exp(v)

    @staticmethod
    def deriv(v):
        return 1.0 / np.asarray(v, np.float64)

    @staticmethod
    def update(v, dv):
        return np.exp(np.log(v) + dv)

    @staticmethod
    def error(v, err):
        """Error in the transformed domain of relative errors ``err``."""
        return np.log1p(np.asarray(err, np.float64))


def smoothness_constraints(mesh, n_params=None):
    """First-order smoothness constraint matrix (CSR rows of +1 / -1) over the
    faces shared by two cells whose markers (parameters) differ and are both
    >= 0, for a mesh whose cell markers are the parameters (no region
    manager; with one, RegionManager.constraintMatrix).  Rows follow the
    shared faces sorted by their node ids."""
    cells = mesh.cells[:, :mesh.dim() + 1].astype(np.int64)
    mk = mesh.cell_markers.astype(np.int64)
    nv = cells.shape[1]
    n = mesh.nodeCount()
    faces, owner = [], []
    for skip in range(nv):
        cols = [j for j in range(nv) if j != skip]
        faces.append(np.sort(cells[:, cols], axis=1))
        owner.append(np.arange(len(cells)))
    faces = np.concatenate(faces)
    owner = np.concatenate(owner)
    key = faces[:, 0]
    for j in range(1, faces.shape[1]):
        key = key * n + faces[:, j]
    order = np.argsort(key, kind="stable")
    key, owner = key[order], owner[order]
    pair = np.nonzero(key[1:] == key[:-1])[0]
    a, b = owner[pair], owner[pair + 1]
    pa, pb = mk[a], mk[b]
    keep = (pa >= 0) & (pb >= 0) & (pa != pb)
    pa, pb = pa[keep], pb[keep]
    P = int(mk.max()) + 1 if n_params is None else int(n_params)
    R = len(pa)
    rowptr = np.arange(0, 2 * R + 1, 2, dtype=np.int32)
    cols = np.empty(2 * R, np.int32)
    vals = np.empty(2 * R)
    lo, hi = np.minimum(pa, pb), np.maximum(pa, pb)
    cols[0::2], cols[1::2] = lo, hi
    vals[0::2], vals[1::2] = 1.0, -1.0
    return rowptr, cols, vals, P


def _transpose_csr(rowptr, cols, vals, ncols):
    import scipy.sparse as sp
    C = sp.csr_matrix((vals, cols, rowptr), shape=(len(rowptr) - 1, ncols))
    T = C.T.tocsr()
    T.sort_indices()
    return T.indptr.astype(np.int32), T.indices.astype(np.int32), T.data.astype(np.float64)


def _torch():
    import torch
    return torch


def cgls(J, C, dweight, b, x0, wc, wm, tm, td, lam, rough, max_iter=200, tol=-1.0):
    """``ertgb_cgls`` on device arrays: J (torch CUDA tensor D x P, FP64 or
    FP32), C = (rowptr, cols, vals, P) host CSR, vectors numpy FP64.
    Returns (x, iterations)."""
    torch = _torch()
    dev = J.device
    D, P = J.shape
    rp, ci, cv, _ = C
    trp, tci, tcv = _transpose_csr(rp, ci, cv, P)

    def d(a, dt=torch.float64):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)

    t = {"crp": d(rp, torch.int32), "cci": d(ci, torch.int32), "cv": d(cv), "trp": d(trp, torch.int32),
         "tci": d(tci, torch.int32), "tcv": d(tcv), "dw": d(dweight), "b": d(b), "x": d(x0), "wc": d(wc),
         "wm": d(wm), "tm": d(tm), "td": d(td), "r": d(rough)}
    it = ctypes.c_int32()
    stream = torch.cuda.current_stream(dev).cuda_stream
    p = lambda k: ctypes.c_void_p(t[k].data_ptr())  # noqa: E731
    lib = _native.load()
    _native.check(None, lib.ertgb_cgls(ctypes.c_void_p(J.data_ptr()), 0 if J.dtype == torch.float64 else 1, D, P,
                                       len(rp) - 1, p("crp"), p("cci"), p("cv"), p("trp"), p("tci"), p("tcv"),
                                       p("dw"), p("b"), p("x"), p("wc"), p("wm"), p("tm"), p("td"), float(lam),
                                       p("r"), int(max_iter), float(tol), ctypes.byref(it), ctypes.c_void_p(stream)))
    torch.cuda.synchronize(dev)
    return t["x"].cpu().numpy(), it.value


class GaussNewton:
    """State of a regularised log-log Gauss-Newton inversion around ``fop``."""

    def __init__(self, fop, data, error, lam=20.0, max_cgls=200, jacobian_dtype="float64", line_search=True):
        self.fop = fop
        self.data = np.asarray(data, np.float64)
        self.error = np.asarray(error, np.float64)
        self.lam = float(lam)
        self.max_cgls = int(max_cgls)
        self.jdtype = jacobian_dtype
        self.line_search = line_search
        self.tD = TransLog
        self.tM = TransLog
        # with a region manager its constraint matrix over the parameter mesh
        # (RegionManager::fillConstraints); on a mesh given as the forward mesh
        # (ignoreRegionManager) first-order rows between its parameter cells
        rm = fop.regionManager() if hasattr(fop, "regionManager") else None
        self.C = rm.constraintMatrix() if rm is not None else smoothness_constraints(fop.mesh(), fop.parameterCount)
        import scipy.sparse as sp
        rp, ci, cv, P = self.C
        self._Cs = sp.csr_matrix((cv, ci, rp), shape=(len(rp) - 1, P))
        self.wc = np.ones(len(self.C[0]) - 1)
        self.wm = np.ones(fop.parameterCount)
        self.dweight = 1.0 / self.tD.error(self.data, self.error)
        self.stats = []

    def _C_mul(self, x):
        return self._Cs @ x

    def roughness(self, model):
        return self._C_mul(self.tM.trans(model) * self.wm) * self.wc

    def phi_d(self, response):
        dd = (self.tD.trans(self.data) - self.tD.trans(response)) * self.dweight
        return float(dd @ dd)

    def phi_m(self, model):
        r = self.roughness(model)
        return float(r @ r)

    def phi(self, model, response):
        return self.phi_d(response) + self.lam * self.phi_m(model)

    def step(self, model, response=None):
        """One step from ``model``; returns (model_new, response_new, info)."""
        fop = self.fop
        if response is None:
            response = fop.response(model)
        J = fop.createJacobian(model, dtype=self.jdtype)
        b = self.tD.trans(self.data) - self.tD.trans(response)
        dm, it = cgls(J, self.C, self.dweight, b, np.zeros_like(model, dtype=np.float64), self.wc, self.wm,
                      self.tM.deriv(model), self.tD.deriv(response), self.lam, self.roughness(model),
                      max_iter=self.max_cgls)
        model_new = self.tM.update(model, dm)
        response_new = fop.response(model_new)
        tau, responses = 1.0, 2
        if self.line_search:
            tau, extra = self._line_search(model, response, model_new, response_new, dm)
            responses += extra
        if tau < 0.95:
            model_new = self.tM.update(model, dm * tau)
            response_new = fop.response(model_new)
            responses += 1
        info = {"cgls_iterations": it, "tau": tau, "phi_before": self.phi(model, response),
                "phi_after": self.phi(model_new, response_new), "phi_d": self.phi_d(response_new),
                "responses": responses}
        self.stats.append(info)
        return model_new, response_new, info

    def _line_search(self, model, response, model_new, response_new, dm):
        """RInversion::linesearch: best of 101 step lengths on the linear
        interpolation of the transformed response, parabolic fit below 0.03.
        With log transforms both the interpolated data and the model are
        linear in tau in the transformed domain, so phi(tau) is a quadratic
        whose three coefficients are computed once (same grid, same minimum)."""
        d_model = self.tM.trans(model_new) - self.tM.trans(model)
        d_data = self.tD.trans(response_new) - self.tD.trans(response)
        dd0 = (self.tD.trans(self.data) - self.tD.trans(response)) * self.dweight
        dd1 = d_data * self.dweight
        r0 = self.roughness(model)
        r1 = self._C_mul(d_model * self.wm) * self.wc
        c0 = dd0 @ dd0 + self.lam * (r0 @ r0)
        c1 = -2.0 * (dd0 @ dd1) + 2.0 * self.lam * (r0 @ r1)
        c2 = dd1 @ dd1 + self.lam * (r1 @ r1)
        min_phi, min_tau = self.phi(model, response), 0.0
        for i in range(1, 101):
            tau = 0.01 * i
            ph = c0 + tau * (c1 + tau * c2)
            if ph < min_phi:
                min_phi, min_tau = ph, tau
        extra = 0
        tau = min_tau
        if tau < 0.03:
            tq = 0.3
            model_q = self.tM.update(model, d_model * tq)
            resp_q = self.fop.response(model_q)
            extra = 1
            phi0 = self.phi(model, response)
            phi10 = self.phi(model_new, response_new) - phi0
            phit0 = self.phi(model_q, resp_q) - phi0
            dphit = phit0 - phi10 * tq
            tau = 0.0 if abs(dphit) < 1e-12 else (phit0 - phi10 * tq * tq) / dphit / 2.0
            tau = min(tau, 1.0)
            tau = max(tau, 0.03)
        return tau, extra
