"""Independent ERT problems solved together on one GPU.

``BatchedERTModelling`` takes any number of set-up ``ERTModelling``
operators (different meshes, electrode counts, schemes, wavenumbers) and
computes all their responses with one batched solve (libertgb's
``ertgb_batch_response``): assembly, right-hand sides and collection run per
problem, the linear systems of every source x wavenumber of every problem go
through one mixed-precision block PCG whose kernels each cover all problems
in a single launch, captured in CUDA graphs, with the tile shape chosen by an
autotuner on the batch itself.  Jacobians then come from each operator
(``createJacobian``) as usual.

pyGIMLi has no batch API: every ``ERTModelling`` solves its own problem
(pygimli/physics/ert/ertModelling.py:73-246); the batch returns exactly what
each operator's ``response`` would (to the solver tolerance).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native


def _torch():
    import torch
    return torch


class BatchedERTModelling:
    def __init__(self, fops):
        self.fops = list(fops)
        if not self.fops:
            raise ValueError("empty batch")
        dev = {f.device for f in self.fops}
        if len(dev) != 1:
            raise ValueError("all operators of a batch must use one device")
        if len({id(f) for f in self.fops}) != len(self.fops):
            raise ValueError("an operator appears twice in the batch")
        self.device = dev.pop()
        self.info = None

    def __len__(self):
        return len(self.fops)

    def response(self, models):
        """Apparent resistivities of every problem (list of numpy arrays, or
        of CUDA tensors when the models are CUDA tensors of per-cell values)."""
        torch = _torch()
        if len(models) != len(self.fops):
            raise ValueError("one model per problem")
        dev = torch.device("cuda", self.device)
        rhos, outs, on_dev = [], [], True
        for f, m in zip(self.fops, models):
            f._ready()
            if isinstance(m, torch.Tensor) and m.is_cuda:
                rho = m.to(torch.float64).contiguous()
                if rho.numel() != f.mesh().cellCount():
                    raise ValueError("device models must be per-cell resistivities")
            else:
                on_dev = False
                a = np.asarray(m, np.float64)
                if np.min(a) < 1e-12:
                    raise ValueError("response for model with negative or zero resistivity is not defined")
                rho = torch.from_numpy(np.ascontiguousarray(f.mapERTModel(a))).to(dev)
            rhos.append(rho)
            outs.append(torch.empty(f._data.size(), dtype=torch.float64, device=dev))
        n = len(self.fops)
        ctxs = (ctypes.c_void_p * n)(*[f._ctx.value for f in self.fops])
        rp = (ctypes.c_void_p * n)(*[r.data_ptr() for r in rhos])
        op = (ctypes.c_void_p * n)(*[o.data_ptr() for o in outs])
        info = _native.BatchInfo()
        lib = _native.load()
        stream = torch.cuda.current_stream(dev).cuda_stream
        _native.check(None, lib.ertgb_batch_response(ctxs, n, rp, op, ctypes.byref(info), ctypes.c_void_p(stream)))
        for f, m, r in zip(self.fops, models, rhos):
            f._last_model = m
        self._rhos = rhos
        self.info = {
            "rows_per_tile": info.rows_per_tile, "rhs_width": info.rhs_width,
            "candidates": [(info.cand_rows[i], info.cand_width[i], info.cand_ms[i]) for i in range(info.n_candidates)],
            "cached": bool(info.cached), "spmm_tiles": info.spmm_tiles, "vector_tiles": info.vector_tiles,
            "columns": info.columns, "iterations": info.iterations, "stalled_columns": info.stalled_columns,
            "launches": info.launches, "ms_assemble": info.ms_assemble, "ms_solve": info.ms_solve,
            "ms_collect": info.ms_collect}
        if on_dev:
            return outs
        torch.cuda.synchronize(dev)
        return [o.cpu().numpy() for o in outs]

    def createJacobian(self, models, dtype="float64"):
        """Jacobians of every problem from the potentials of the last batched
        response (list of device tensors)."""
        return [f.createJacobian(m, dtype=dtype) for f, m in zip(self.fops, models)]
