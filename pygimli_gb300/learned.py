"""Learned preconditioner of the mixed-precision block PCG: weights,
training loop, persistence.

The network (4 message-passing layers of width 64 on the graph of the system
matrix; kernels in csrc/learned.cu) emits the factor G of M^-1 = G^T G as a
correction of the Jacobi factor,

    G_ii = exp(tanh(delta_ii)) / sqrt(A_ii),   G_ij = delta_ij / sqrt(A_jj)  (j < i),

so G^T G is SPD for any weights and a zero decoder is plain Jacobi.  It is
trained on the GPU by the library's own forward and backward kernels: for
each training model the library assembles the system matrices of every
wavenumber (the method's FP64 assembly) and returns Kaporin's condition
number of G A G^T (exact; its minimiser on this pattern is FSAI) with its
gradient; an Adam kernel updates the FP32 weights.  The method's FP64 solves
judge the result: PCG iterations to the FP64 true-residual tolerance on
held-out models, with the FP64 Jacobi solver as the fallback of stalled
columns, so the converged accuracy does not depend on the network.

Nothing here exists in pyGIMLi (it factors each system with CHOLMOD,
core/src/bert/dcfemmodelling.cpp:2199-2210).
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _native

NPARAM = _native.LP_NPARAM
HIDDEN = 64
LAYERS = 4
NFEAT = 4


def layout():
    """(name, shape) of the blocks of the flat FP32 weight vector, in order."""
    H = HIDDEN
    out = [("enc_n_W", (H, NFEAT)), ("enc_n_b", (H,)), ("enc_e_W", (H, NFEAT)), ("enc_e_b", (H,))]
    for l in range(LAYERS):
        out += [(f"W1_{l}", (H, 3 * H)), (f"b1_{l}", (H,)), (f"W2_{l}", (H, 2 * H)), (f"b2_{l}", (H,))]
    out += [("wo", (H,)), ("bo", (1,)), ("wd", (H,)), ("bd", (1,))]
    return out


def init_weights(seed=0):
    """He-normal encoder and layer weights (layers at half scale for the
    residual updates), zero biases and a zero decoder: G starts as Jacobi."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in layout():
        if name in ("enc_n_W", "enc_e_W"):
            parts.append(rng.normal(0.0, np.sqrt(2.0 / shape[1]), shape))
        elif name.startswith(("W1_", "W2_")):
            parts.append(rng.normal(0.0, 0.5 * np.sqrt(2.0 / shape[1]), shape))
        else:
            parts.append(np.zeros(shape))
    w = np.concatenate([p.ravel() for p in parts]).astype(np.float32)
    assert w.size == NPARAM
    return w


def _torch():
    import torch
    return torch


class LearnedPreconditioner:
    """Weights of the network plus the training loop."""

    def __init__(self, weights=None, seed=0):
        self.weights = init_weights(seed) if weights is None else np.ascontiguousarray(weights, np.float32)
        if self.weights.size != NPARAM:
            raise ValueError(f"expected {NPARAM} weights, got {self.weights.size}")
        self.history = []

    # ------------------------------------------------------------ storage
    def save(self, path, **meta):
        np.savez_compressed(path, weights=self.weights, **{k: np.asarray(v) for k, v in meta.items()})

    @classmethod
    def load(cls, path):
        z = np.load(path)
        obj = cls(z["weights"])
        obj.meta = {k: z[k] for k in z.files if k != "weights"}
        return obj

    # ----------------------------------------------------------- training
    def train(self, fop, models, steps, lr=1e-3, clip=1.0, betas=(0.9, 0.999), eps=1e-8, log_every=0,
              tasks=None, lr_final=None):
        """Adam on Kaporin's number over ``models`` (per-cell or per-parameter
        resistivities of ``fop``'s mesh), cycling through them for ``steps``
        steps; every step assembles one model's matrices (all wavenumbers).
        ``tasks`` = [(fop, models), ...] trains over several meshes in turn
        (then ``fop`` and ``models`` are ignored).  The learning rate decays
        geometrically to ``lr_final`` (default: constant).  Returns the list of
        (step, loss)."""
        torch = _torch()
        tasks = tasks if tasks is not None else [(fop, models)]
        fop = tasks[0][0]
        dev = torch.device("cuda", fop.device)
        theta = torch.from_numpy(self.weights.copy()).to(dev)
        grad = torch.zeros_like(theta)
        m = torch.zeros_like(theta)
        v = torch.zeros_like(theta)
        lib = _native.load()
        hist = []
        t0 = time.time()
        decay = 1.0 if not lr_final else (lr_final / lr) ** (1.0 / max(1, steps - 1))
        for step in range(1, steps + 1):
            fop, models = tasks[(step - 1) % len(tasks)]
            fop.assemble(models[((step - 1) // len(tasks)) % len(models)])
            loss = fop.lpLossGrad(theta, grad)
            lr_s = lr * decay ** (step - 1)
            stream = torch.cuda.current_stream(dev).cuda_stream
            _native.check(None, lib.ertgb_lp_adam(ctypes.c_void_p(theta.data_ptr()), ctypes.c_void_p(grad.data_ptr()),
                                                  ctypes.c_void_p(m.data_ptr()), ctypes.c_void_p(v.data_ptr()),
                                                  NPARAM, lr_s, betas[0], betas[1], eps, step, clip,
                                                  ctypes.c_void_p(stream)))
            hist.append((step, loss))
            if log_every and step % log_every == 0:
                print(f"step {step} loss {loss:.5f} ({time.time() - t0:.1f} s)", flush=True)
        torch.cuda.synchronize(dev)
        self.weights = theta.cpu().numpy()
        self.history += hist
        return hist

    def loss(self, fop, model):
        """Kaporin's number (mean over wavenumbers) of ``model``'s matrices."""
        torch = _torch()
        theta = torch.from_numpy(self.weights).to(torch.device("cuda", fop.device))
        fop.assemble(model)
        return fop.lpLossGrad(theta, None)
