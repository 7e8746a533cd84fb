// Incomplete Cholesky IC(0) preconditioner of the FP64 block PCG.
//
// M = L L^T with L on the lower triangle of A's own pattern (no fill), the
// factor of each wavenumber's system matrix computed on the device after
// assembly, M^-1 r applied to all columns by a forward and a backward
// triangular solve.  Rows depend on earlier rows only through the pattern,
// so both the factorization and the solves run level by level (level of a
// row = 1 + the largest level of the rows it depends on), one launch per
// level, all rows of a level in parallel: one thread per (row, wavenumber)
// in the factorization, one warp per (row, 32 right-hand sides) in the
// solves.
//
// Factor (row-oriented, rows in level order): for j < i in row i
//   L_ij = (A_ij - sum_{k < j} L_ik L_jk) / L_jj,   L_ii = sqrt(A_ii - sum_k L_ik^2),
// the sums over the common columns of rows i and j in ascending order.  A
// pivot that is not positive (IC(0) need not exist for a matrix that is not
// an M-matrix) is replaced by A_ii and counted.
//
// This is the preconditioner the reference's CHOLMOD factorization would be
// without fill (core/src/cholmodWrapper.cpp:309-420 factors A exactly); it
// serves as the incomplete-factorization option beside Jacobi of the plain
// FP64 solver.
#include <algorithm>
#include <cmath>

#include "ertgb_internal.cuh"

namespace ertgb {

namespace {

__global__ void k_ic0_factor(int nrow, const int32_t *__restrict__ rows, int nK, int64_t nnz, int64_t nL,
                             const int32_t *__restrict__ Lrp, const int32_t *__restrict__ Lci,
                             const int32_t *__restrict__ LtoA, const double *__restrict__ A, double *__restrict__ L,
                             int32_t *__restrict__ bad) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= (int64_t)nrow * nK) return;
    const int ki = (int)(idx / nrow);
    const int32_t i = rows[idx - (int64_t)ki * nrow];
    const double *Ak = A + ki * nnz;
    double *Lk = L + ki * nL;
    const int32_t q0 = Lrp[i], qd = Lrp[i + 1] - 1;  // the diagonal closes the row
    for (int32_t q = q0; q < qd; q++) {
        const int32_t j = Lci[q];
        double s = Ak[LtoA[q]];
        int32_t a = q0, b = Lrp[j];
        const int32_t be = Lrp[j + 1] - 1;
        while (a < q && b < be) {
            const int32_t ca = Lci[a], cb = Lci[b];
            if (ca == cb) {
                s -= Lk[a] * Lk[b];
                a++;
                b++;
            } else if (ca < cb) {
                a++;
            } else {
                b++;
            }
        }
        Lk[q] = s / Lk[be];
    }
    const double aii = Ak[LtoA[qd]];
    double d = aii;
    for (int32_t q = q0; q < qd; q++) d -= Lk[q] * Lk[q];
    if (!(d > 0.0) || !isfinite(d)) {
        d = aii;
        atomicAdd(bad, 1);
    }
    Lk[qd] = sqrt(d);
}

// z_i = (r_i - sum_{j < i} L_ij z_j) / L_ii for the rows of one level: one
// warp per (row, 32-column chunk)
__global__ void k_ic0_fwd(int nrow, const int32_t *__restrict__ rows, int64_t Rpad, int nE, int64_t R, int64_t nL,
                          const int32_t *__restrict__ Lrp, const int32_t *__restrict__ Lci,
                          const double *__restrict__ L, const double *__restrict__ r, double *__restrict__ z) {
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nch = Rpad / 32;
    if (warp >= (int64_t)nrow * nch) return;
    const int32_t i = rows[warp / nch];
    const int64_t t = (warp % nch) * 32 + (threadIdx.x & 31);
    const int32_t q0 = Lrp[i], qd = Lrp[i + 1] - 1;
    const double *Lk = L + (t < R ? t / nE : 0) * nL;
    double s = r[(int64_t)i * Rpad + t];
#pragma unroll 8
    for (int32_t q = q0; q < qd; q++) s -= Lk[q] * z[(int64_t)Lci[q] * Rpad + t];
    z[(int64_t)i * Rpad + t] = s / Lk[qd];
}

// z_i = (z_i - sum_{j > i} L_ji z_j) / L_ii, in place, for the rows of one
// level of the transposed pattern (U row i: the diagonal, then j > i): one
// warp per (row, 32-column chunk)
__global__ void k_ic0_bwd(int nrow, const int32_t *__restrict__ rows, int64_t Rpad, int nE, int64_t R, int64_t nL,
                          const int32_t *__restrict__ Urp, const int32_t *__restrict__ Uci,
                          const int32_t *__restrict__ UtoL, const double *__restrict__ L, double *__restrict__ z) {
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nch = Rpad / 32;
    if (warp >= (int64_t)nrow * nch) return;
    const int32_t i = rows[warp / nch];
    const int64_t t = (warp % nch) * 32 + (threadIdx.x & 31);
    const int32_t q0 = Urp[i], q1 = Urp[i + 1];
    const double *Lk = L + (t < R ? t / nE : 0) * nL;
    double s = z[(int64_t)i * Rpad + t];
#pragma unroll 8
    for (int32_t q = q0 + 1; q < q1; q++) s -= Lk[UtoL[q]] * z[(int64_t)Uci[q] * Rpad + t];
    z[(int64_t)i * Rpad + t] = s / Lk[UtoL[q0]];
}

// rows ordered by level: level(i) = 1 + max level(dep) over the rows i
// depends on (dep(i) = columns < i of the lower row, or > i of the upper row)
void level_order(int64_t n, const std::vector<int32_t> &rp, const std::vector<int32_t> &ci, bool lower,
                 std::vector<int32_t> &order, std::vector<int32_t> &lptr) {
    std::vector<int32_t> lev((size_t)n, 0);
    int32_t nlev = 0;
    for (int64_t s = 0; s < n; s++) {
        const int64_t i = lower ? s : n - 1 - s;
        int32_t l = 0;
        for (int32_t q = rp[i]; q < rp[i + 1]; q++) {
            const int32_t j = ci[q];
            if (lower ? j < i : j > i) l = std::max(l, lev[j] + 1);
        }
        lev[i] = l;
        nlev = std::max(nlev, l + 1);
    }
    lptr.assign((size_t)nlev + 1, 0);
    for (int64_t i = 0; i < n; i++) lptr[lev[i] + 1]++;
    for (int32_t l = 0; l < nlev; l++) lptr[l + 1] += lptr[l];
    order.assign((size_t)n, 0);
    std::vector<int32_t> pos(lptr.begin(), lptr.end() - 1);
    for (int64_t i = 0; i < n; i++) order[pos[lev[i]]++] = (int32_t)i;
}

}  // namespace

void ic0_setup(Context &c, cudaStream_t s) {
    MeshData &m = c.mesh;
    Ic0Plan &P = m.ic0;
    if (!P.ready) {
        level_order(m.n, m.Lrowptr, m.Lcolidx, true, P.frow, P.flev);
        level_order(m.n, m.Urowptr, m.Ucolidx, false, P.brow, P.blev);
        P.d_frow.upload(P.frow, s);
        P.d_brow.upload(P.brow, s);
        P.ready = true;
    }
    const int64_t nL = (int64_t)m.Lcolidx.size();
    c.d_ic.alloc((size_t)c.nK * nL);
    DBuf<int32_t> &bad = c.d_ic_bad;
    bad.alloc(1);
    bad.zero(s);
    const int nlev = (int)P.flev.size() - 1;
    for (int l = 0; l < nlev; l++) {
        const int a = P.flev[l], nrow = P.flev[l + 1] - a;
        const int64_t th = (int64_t)nrow * c.nK;
        k_ic0_factor<<<(unsigned)ceil_div(th, 128), 128, 0, s>>>(nrow, P.d_frow.p + a, c.nK, m.nnz, nL,
                                                                 m.d_Lrowptr.p, m.d_Lcolidx.p, m.d_LtoA.p, c.d_S.p,
                                                                 c.d_ic.p, bad.p);
    }
    ERTGB_CUDA(cudaGetLastError());
    int32_t h = 0;
    ERTGB_CUDA(cudaMemcpyAsync(&h, bad.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    c.ic0_breakdowns = h;
    c.stats.launches_response += nlev;
}

void ic0_apply(Context &c, const double *r, double *z, cudaStream_t s) {
    MeshData &m = c.mesh;
    Ic0Plan &P = m.ic0;
    const int64_t nL = (int64_t)m.Lcolidx.size();
    const int nf = (int)P.flev.size() - 1, nb = (int)P.blev.size() - 1;
    for (int l = 0; l < nf; l++) {
        const int a = P.flev[l], nrow = P.flev[l + 1] - a;
        k_ic0_fwd<<<(unsigned)ceil_div((int64_t)nrow * (c.Rpad / 32), 8), 256, 0, s>>>(
            nrow, P.d_frow.p + a, c.Rpad, c.nE, c.R, nL, m.d_Lrowptr.p, m.d_Lcolidx.p, c.d_ic.p, r, z);
    }
    for (int l = 0; l < nb; l++) {
        const int a = P.blev[l], nrow = P.blev[l + 1] - a;
        k_ic0_bwd<<<(unsigned)ceil_div((int64_t)nrow * (c.Rpad / 32), 8), 256, 0, s>>>(
            nrow, P.d_brow.p + a, c.Rpad, c.nE, c.R, nL, m.d_Urowptr.p, m.d_Ucolidx.p, m.d_UtoL.p, c.d_ic.p, z);
    }
    ERTGB_CUDA(cudaGetLastError());
}

int ic0_launches(const Context &c) {
    const Ic0Plan &P = c.mesh.ic0;
    return (int)(P.flev.size() - 1 + P.blev.size() - 1);
}

}  // namespace ertgb
