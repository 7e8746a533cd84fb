"""Test infrastructure only: FP64 restatement of the learned preconditioner
and of its training loss and gradients.

The preconditioner is M^-1 = G^T G with G lower triangular on the lower
pattern of the system matrix A.  A message-passing network on the graph of
A (nodes = rows, edges = stored entries, diagonal included) emits one
number delta per entry of G, a correction of the Jacobi factor D^-1/2:

    G_ii = exp(CLAMP * tanh(delta_ii)) / sqrt(A_ii)
    G_ij = delta_ij / sqrt(A_jj)                      (j < i)

The diagonal of G stays positive, so G is nonsingular and G^T G is SPD for
any network output; a zero decoder gives Jacobi.

Inputs are invariant to a common scaling of A: with Ahat = D^-1/2 A D^-1/2,
edge features f_q = [Ahat_ij, (Ahat^2)_ij, log(A_ii / A_jj), [i == j]] and
node features x_i = [sum_j!=i |Ahat_ij|, deg_i / 16, (Ahat^2)_ii,
sum_j!=i Ahat_ij].

Network (hidden width 64, 4 layers):
    h_i = relu(Wn x_i + bn),  e_q = relu(We f_q + be)           encoders
    per layer:
      z_q = W1 [h_i; h_j; e_q] + b1,  m_q = relu(z_q),  e_q += m_q
      a_i = mean_{q in row i} m_q
      y_i = W2 [h_i; a_i] + b2,  h_i += relu(y_i)
    delta_q = wo . e_q + bo (lower off-diagonal q),  delta_ii = wd . h_i + bd

Training loss: Kaporin's condition number of G A G^T (I. E. Kaporin, "New
convergence results and preconditioning strategies for the conjugate
gradient method", Numer. Linear Algebra Appl. 1, 1994), per matrix and up
to the constant log det A:
    K = log(sum_i q_i / n) - (2/n) sum_i log G_ii,   q_i = (G A G^T)_ii
It is exact (no probe vectors), invariant to the scale of A and of G, and
on a fixed pattern its minimiser is the FSAI factor (``fsai``), which is
the ceiling the network approaches.

There is no counterpart in pyGIMLi (it factors each system with CHOLMOD,
core/src/bert/dcfemmodelling.cpp:2199-2210): the GPU kernels of
pygimli_gb300/csrc/learned.cu are checked against this file, and this file
against central finite differences.
"""
from __future__ import annotations

import numpy as np

HIDDEN = 64
LAYERS = 4
NFEAT = 4
CLAMP = 1.0
FSAI_MAX_ROW = 24


def param_layout():
    """(name, shape) in the order of the flat FP32 parameter vector."""
    H = HIDDEN
    L = [("enc_n_W", (H, NFEAT)), ("enc_n_b", (H,)), ("enc_e_W", (H, NFEAT)), ("enc_e_b", (H,))]
    for l in range(LAYERS):
        L += [(f"W1_{l}", (H, 3 * H)), (f"b1_{l}", (H,)), (f"W2_{l}", (H, 2 * H)), (f"b2_{l}", (H,))]
    L += [("wo", (H,)), ("bo", (1,)), ("wd", (H,)), ("bd", (1,))]
    return L


def param_count():
    return int(sum(np.prod(s) for _, s in param_layout()))


def unflatten(theta):
    out, o = {}, 0
    for name, shape in param_layout():
        n = int(np.prod(shape))
        out[name] = np.asarray(theta[o:o + n], np.float64).reshape(shape)
        o += n
    return out


def flatten(P):
    return np.concatenate([np.asarray(P[name], np.float64).ravel() for name, _ in param_layout()])


def init_params(seed=0, decoder_scale=0.0):
    """He-normal weights, zero biases; a zero decoder makes G the Jacobi factor."""
    rng = np.random.default_rng(seed)
    P = {}
    for name, shape in param_layout():
        if name.startswith(("enc_n_W", "enc_e_W")):
            P[name] = rng.normal(0.0, np.sqrt(2.0 / shape[1]), shape)
        elif name.startswith("W1_") or name.startswith("W2_"):
            P[name] = rng.normal(0.0, 0.5 * np.sqrt(2.0 / shape[1]), shape)
        elif name in ("wo", "wd"):
            P[name] = rng.normal(0.0, decoder_scale, shape) if decoder_scale else np.zeros(shape)
        else:
            P[name] = np.zeros(shape)
    return flatten(P)


class Graph:
    """Graph of a CSR matrix with symmetric pattern and sorted columns."""

    def __init__(self, rowptr, cols):
        self.rowptr = np.asarray(rowptr, np.int64)
        self.cols = np.asarray(cols, np.int64)
        n = len(self.rowptr) - 1
        self.n = n
        self.E = len(self.cols)
        self.deg = np.diff(self.rowptr)
        self.row = np.repeat(np.arange(n), self.deg)
        key = self.row * n + self.cols
        tkey = self.cols * n + self.row
        order = np.argsort(key)
        self.T = order[np.searchsorted(key[order], tkey)]
        assert np.array_equal(self.cols[self.T], self.row)
        lower = self.cols <= self.row
        self.lq = np.nonzero(lower)[0]                     # full index of each G entry (row-major)
        self.Lrow = self.row[self.lq]
        self.Lcol = self.cols[self.lq]
        self.Lrowptr = np.concatenate([[0], np.cumsum(np.bincount(self.Lrow, minlength=n))])
        self.dq = np.nonzero(self.cols == self.row)[0]
        assert len(self.dq) == n
        self.Ldiag = self.Lcol == self.Lrow


def segsum(v, idx, n):
    out = np.zeros((n,) + v.shape[1:])
    np.add.at(out, idx, v)
    return out


def fsai(g, A):
    """FSAI factor on the lower pattern (values in G-entry order); rows longer
    than FSAI_MAX_ROW or not positive definite fall back to 1/sqrt(A_ii)."""
    GL = np.zeros(len(g.lq))
    for i in range(g.n):
        p0, p1 = g.Lrowptr[i], g.Lrowptr[i + 1]
        S = g.Lcol[p0:p1]
        m = len(S)
        ok = m <= FSAI_MAX_ROW
        if ok:
            M = np.zeros((m, m))
            for a, ra in enumerate(S):
                q0, q1 = g.rowptr[ra], g.rowptr[ra + 1]
                pos = np.searchsorted(g.cols[q0:q1], S)
                hit = (pos < q1 - q0)
                hit[hit] &= g.cols[q0:q1][pos[hit]] == S[hit]
                M[a, hit] = A[q0 + pos[hit]]
            try:
                Lc = np.linalg.cholesky(M)
            except np.linalg.LinAlgError:
                ok = False
        if ok:
            e = np.zeros(m)
            e[-1] = 1.0
            y = np.linalg.solve(M, e)
            GL[p0:p1] = y / np.sqrt(y[-1])
        else:
            GL[p0:p1 - 1] = 0.0
            GL[p1 - 1] = 1.0 / np.sqrt(A[g.dq[i]])
    return GL


def a2_edges(g, ahat):
    """(Ahat^2)_ij for every stored entry (i, j): merge of rows i and j."""
    import scipy.sparse as sp
    Ah = sp.csr_matrix((ahat, g.cols, g.rowptr), shape=(g.n, g.n))
    A2 = (Ah @ Ah).tocsr()
    return np.asarray(A2[g.row, g.cols]).ravel()


def features(g, A):
    """Node features x (n x 4), edge features f (E x 4)."""
    d = A[g.dq]
    dr, dc = d[g.row], d[g.cols]
    ahat = A / np.sqrt(dr * dc)
    a2 = a2_edges(g, ahat)
    isd = (g.row == g.cols).astype(np.float64)
    off = 1.0 - isd
    f = np.stack([ahat, a2, np.log(dr / dc), isd], axis=1)
    x = np.stack([segsum(np.abs(ahat) * off, g.row, g.n), g.deg / 16.0, a2[g.dq],
                  segsum(ahat * off, g.row, g.n)], axis=1)
    return x, f


def relu(v):
    return np.maximum(v, 0.0)


def forward(theta, g, x, f, A):
    P = unflatten(theta)
    c = {"pre_h": x @ P["enc_n_W"].T + P["enc_n_b"], "pre_e": f @ P["enc_e_W"].T + P["enc_e_b"]}
    h = relu(c["pre_h"])
    e = relu(c["pre_e"])
    layers = []
    for l in range(LAYERS):
        X = np.concatenate([h[g.row], h[g.cols], e], axis=1)
        z = X @ P[f"W1_{l}"].T + P[f"b1_{l}"]
        m = relu(z)
        a = segsum(m, g.row, g.n) / g.deg[:, None]
        y = np.concatenate([h, a], axis=1) @ P[f"W2_{l}"].T + P[f"b2_{l}"]
        layers.append((h, e, z, a, y))
        e = e + m
        h = h + relu(y)
    c["layers"], c["h"], c["e"] = layers, h, e
    dl = e[g.lq] @ P["wo"] + P["bo"][0]
    dd = h @ P["wd"] + P["bd"][0]
    delta = np.where(g.Ldiag, dd[g.Lrow], dl)
    c["delta"] = delta
    dsq = 1.0 / np.sqrt(A[g.dq])
    G = np.where(g.Ldiag, np.exp(CLAMP * np.tanh(delta)) * dsq[g.Lrow], delta * dsq[g.Lcol])
    return G, c


def kaporin(g, A, G):
    """K (up to log det A) and dK/dG per G entry."""
    gA = np.zeros(len(G))          # (A g_i)_a for every entry (i, a) of G
    Ad = {}
    for q in range(g.E):
        Ad[(g.row[q], g.cols[q])] = A[q]
    for i in range(g.n):
        p0, p1 = g.Lrowptr[i], g.Lrowptr[i + 1]
        S = g.Lcol[p0:p1]
        for a_, a in enumerate(S):
            gA[p0 + a_] = sum(Ad.get((a, b), 0.0) * G[p0 + b_] for b_, b in enumerate(S))
    q = segsum(G * gA, g.Lrow, g.n)
    Q = np.sum(q)
    Gd = G[g.Ldiag]
    K = float(np.log(Q / g.n) - 2.0 * np.mean(np.log(Gd)))
    dG = 2.0 * gA / Q
    dG[g.Ldiag] -= 2.0 / (g.n * Gd)
    return K, dG


def backward(theta, g, x, f, A, G, c, dG):
    P = unflatten(theta)
    D = {name: np.zeros(shape) for name, shape in param_layout()}
    t = np.tanh(c["delta"])
    dsq = 1.0 / np.sqrt(A[g.dq])
    dd = np.where(g.Ldiag, dG * G * CLAMP * (1.0 - t * t), dG * dsq[g.Lcol])
    off = ~g.Ldiag
    eL, hL = c["e"], c["h"]
    D["wo"] = eL[g.lq[off]].T @ dd[off]
    D["bo"][0] = np.sum(dd[off])
    ddiag = np.zeros(g.n)
    ddiag[g.Lrow[g.Ldiag]] = dd[g.Ldiag]
    D["wd"] = hL.T @ ddiag
    D["bd"][0] = np.sum(ddiag)
    de = np.zeros((g.E, HIDDEN))
    de[g.lq[off]] = dd[off][:, None] * P["wo"][None, :]
    dh = ddiag[:, None] * P["wd"][None, :]
    for l in reversed(range(LAYERS)):
        h, e, z, a, y = c["layers"][l]
        dy = dh * (y > 0)
        Y = np.concatenate([h, a], axis=1)
        D[f"W2_{l}"] = dy.T @ Y
        D[f"b2_{l}"] = dy.sum(axis=0)
        dY = dy @ P[f"W2_{l}"]
        dh_prev = dh + dY[:, :HIDDEN]
        da = dY[:, HIDDEN:]
        dm = de + (da / g.deg[:, None])[g.row]
        dz = dm * (z > 0)
        X = np.concatenate([h[g.row], h[g.cols], e], axis=1)
        D[f"W1_{l}"] = dz.T @ X
        D[f"b1_{l}"] = dz.sum(axis=0)
        dX = dz @ P[f"W1_{l}"]
        dh_prev += segsum(dX[:, :HIDDEN], g.row, g.n) + segsum(dX[:, HIDDEN:2 * HIDDEN], g.cols, g.n)
        de = de + dX[:, 2 * HIDDEN:]
        dh = dh_prev
    dph = dh * (c["pre_h"] > 0)
    D["enc_n_W"] = dph.T @ x
    D["enc_n_b"] = dph.sum(axis=0)
    dpe = de * (c["pre_e"] > 0)
    D["enc_e_W"] = dpe.T @ f
    D["enc_e_b"] = dpe.sum(axis=0)
    return flatten(D)


def loss_and_grad(theta, g, A, feats=None):
    """Kaporin loss, its gradient in the parameters, and G, for one matrix."""
    x, f = features(g, A) if feats is None else feats
    G, c = forward(theta, g, x, f, A)
    K, dG = kaporin(g, A, G)
    return K, backward(theta, g, x, f, A, G, c, dG), G
