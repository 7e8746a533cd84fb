// Factorized sparse approximate inverse (FSAI) preconditioner, M^-1 = G^T G.
//
// G is lower triangular on the lower-triangular pattern of A.  Row i of G
// solves the small dense SPD system A[S_i, S_i] g = e_i on its pattern
// S_i = { j <= i : A_ij != 0 } and is scaled so that (G A G^T)_ii = 1
// (Kolotilina & Yeremin, "Factorized sparse approximate inverse
// preconditionings I", SIAM J. Matrix Anal. Appl. 14, 1993).  Every row is
// independent: one thread per (row, wavenumber) gathers the submatrix from the
// CSR system matrix, factors it with a dense Cholesky in FP64 and writes its
// row of G.  Rows longer than kMaxRow, or whose submatrix is not numerically
// positive definite, fall back to the Jacobi row 1/sqrt(A_ii).  Applying the
// preconditioner is two parallel sparse products (G, then G^T), no
// triangular solves.
#include <algorithm>
#include <cmath>

#include "ertgb_internal.cuh"

namespace ertgb {

namespace {

constexpr int kMaxRow = 24;  // covers every lower row of P1 and P2 (Tet10) patterns

__device__ inline double csr_get(const int32_t *__restrict__ rowptr, const int32_t *__restrict__ colidx,
                                 const double *__restrict__ vals, int32_t r, int32_t c) {
    int32_t lo = rowptr[r], hi = rowptr[r + 1] - 1;
    while (lo <= hi) {
        const int32_t mid = (lo + hi) >> 1;
        const int32_t v = colidx[mid];
        if (v == c) return vals[mid];
        if (v < c) lo = mid + 1;
        else hi = mid - 1;
    }
    return 0.0;
}

__global__ void k_fsai_setup(int64_t n, int nK, int64_t nnz, int64_t nL, const int32_t *__restrict__ rowptr,
                             const int32_t *__restrict__ colidx, const double *__restrict__ A,
                             const int32_t *__restrict__ Lrowptr, const int32_t *__restrict__ Lcolidx,
                             double *__restrict__ G, int32_t *__restrict__ nfallback) {
    double M[kMaxRow][kMaxRow];
    int32_t S[kMaxRow];
    const int64_t total = n * nK;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ki = t / n;
        const int32_t i = (int32_t)(t - ki * n);
        const double *Ak = A + ki * nnz;
        double *Gk = G + ki * nL;
        const int32_t q0 = Lrowptr[i];
        const int m = Lrowptr[i + 1] - q0;
        bool ok = m <= kMaxRow;
        if (ok) {
            for (int a = 0; a < m; a++) S[a] = Lcolidx[q0 + a];
            // gather the lower triangle of A[S, S] and factor it (Cholesky)
            for (int a = 0; a < m; a++)
                for (int b = 0; b <= a; b++) M[a][b] = csr_get(rowptr, colidx, Ak, S[a], S[b]);
            for (int j = 0; j < m && ok; j++) {
                double d = M[j][j];
                for (int k = 0; k < j; k++) d -= M[j][k] * M[j][k];
                if (!(d > 0.0)) {
                    ok = false;
                    break;
                }
                const double ljj = sqrt(d);
                M[j][j] = ljj;
                for (int a = j + 1; a < m; a++) {
                    double v = M[a][j];
                    for (int k = 0; k < j; k++) v -= M[a][k] * M[j][k];
                    M[a][j] = v / ljj;
                }
            }
        }
        if (ok) {
            // A_S y = e_m: forward substitution gives w = e_m / L_mm; back
            // substitution with L^T; then g = y / sqrt(y_m) = y * L_mm
            double y[kMaxRow];
            const double lmm = M[m - 1][m - 1];
            y[m - 1] = 1.0 / (lmm * lmm);
            for (int j = m - 2; j >= 0; j--) {
                double v = 0.0;
                for (int k = j + 1; k < m; k++) v -= M[k][j] * y[k];
                y[j] = v / M[j][j];
            }
            for (int a = 0; a < m; a++) Gk[q0 + a] = y[a] * lmm;
        } else {
            atomicAdd(nfallback, 1);
            for (int a = 0; a < m - 1; a++) Gk[q0 + a] = 0.0;
            Gk[q0 + m - 1] = 1.0 / sqrt(csr_get(rowptr, colidx, Ak, i, i));
        }
    }
}

// FP32 copies of G and of G^T (gathered through the transpose map)
__global__ void k_fsai_f32(int64_t nL, int nK, const double *__restrict__ G, const int32_t *__restrict__ UtoL,
                           float *__restrict__ G32, float *__restrict__ GT32) {
    const int64_t total = nL * nK;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ki = t / nL, q = t - ki * nL;
        G32[t] = (float)G[t];
        GT32[t] = (float)G[ki * nL + UtoL[q]];
    }
}

}  // namespace

void fsai_setup(Context &c, cudaStream_t s) {
    MeshData &m = c.mesh;
    const int64_t nL = (int64_t)m.Lcolidx.size();
    c.d_G.alloc((size_t)c.nK * nL);
    c.d_G32.alloc((size_t)c.nK * nL);
    c.d_GT32.alloc((size_t)c.nK * nL);
    DBuf<int32_t> fb;
    fb.alloc(1);
    fb.zero(s);
    const int64_t total = m.n * c.nK;
    k_fsai_setup<<<(unsigned)std::min<int64_t>(ceil_div(total, 128), 65535), 128, 0, s>>>(
        m.n, c.nK, m.nnz, nL, m.d_rowptr.p, m.d_colidx.p, c.d_S.p, m.d_Lrowptr.p, m.d_Lcolidx.p, c.d_G.p, fb.p);
    ERTGB_CUDA(cudaGetLastError());
    k_fsai_f32<<<(unsigned)std::min<int64_t>(ceil_div(nL * c.nK, 256), 65535), 256, 0, s>>>(nL, c.nK, c.d_G.p,
                                                                                           m.d_UtoL.p, c.d_G32.p,
                                                                                           c.d_GT32.p);
    ERTGB_CUDA(cudaGetLastError());
    ERTGB_CUDA(cudaMemcpyAsync(&c.fsai_fallback_rows, fb.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    c.stats.launches_response += 2;
}

}  // namespace ertgb
