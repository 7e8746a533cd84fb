// Banded direct solve of the FP64 system matrices (the 2.5-D path).
//
// The reference factors every wavenumber's matrix with CHOLMOD and solves
// each current source with the factor (core/src/bert/dcfemmodelling.cpp:
// 2199-2210, core/src/cholmodWrapper.cpp:309-420).  The 2-D meshes of the
// 2.5-D path have a small bandwidth in their own node order (the para
// meshes: 17-28; otherwise reverse Cuthill-McKee is used when it is
// smaller), so the exact Cholesky factor L of A (L L^T = A, no pivoting, A
// SPD) fits a band of b+1 diagonals and costs n b^2 / 2 multiply-adds:
//
//   band storage, column-major by diagonal: B[j (b+1) + d] = L(j+d, j),
//   one block per wavenumber factors column by column (right-looking):
//     L(j,j) = sqrt(a_jj);  L(j+i,j) = a_{j+i,j} / L(j,j);
//     a_{j+i, j+l} -= L(j+i,j) L(j+l,j)   (1 <= l <= i <= b),
//   then L y = b, L^T x = y for every column of the wavenumber (one thread
//   per right-hand side, sequential over the band; for bandwidths up to 64
//   the last b solution values stay in registers).  Bandwidths up to 31 are
//   factored by one warp per wavenumber (lane d holds L(j+d, j)).
//
// Rows are visited in the chosen order through a permutation, so the
// right-hand-side and solution blocks stay in the mesh's node order.  A pivot
// that is not positive stops the solve with an error (A must be SPD).
#include <algorithm>
#include <cmath>
#include <queue>

#include "ertgb_internal.cuh"

namespace ertgb {

namespace {

constexpr int kBandThreads = 256;

__global__ void __launch_bounds__(kBandThreads) k_band_fill(int64_t n, int b, int nK, int64_t nnz,
                                                             const int32_t *__restrict__ rowptr,
                                                             const int32_t *__restrict__ colidx,
                                                             const int32_t *__restrict__ pos,
                                                             const double *__restrict__ S, double *__restrict__ B) {
    const int64_t total = n * nK;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t / n, i = t - k * n;
        const int64_t pi = pos[i];
        double *Bk = B + k * n * (b + 1);
        for (int32_t s = rowptr[i]; s < rowptr[i + 1]; s++) {
            const int64_t pj = pos[colidx[s]];
            if (pj <= pi) Bk[pj * (b + 1) + (pi - pj)] = S[k * nnz + s];
        }
    }
}

// one block per wavenumber: the band Cholesky factor in place
__global__ void __launch_bounds__(kBandThreads) k_band_factor(int64_t n, int b, double *__restrict__ B,
                                                               int32_t *__restrict__ bad) {
    __shared__ double col[kMaxBand + 1];
    double *A = B + (int64_t)blockIdx.x * n * (b + 1);
    const int tid = threadIdx.x;
    for (int64_t j = 0; j < n; j++) {
        const int m = (int)(n - 1 - j < (int64_t)b ? n - 1 - j : (int64_t)b);
        double *Aj = A + j * (b + 1);
        if (tid == 0) {
            double d = Aj[0];
            if (!(d > 0.0) || !isfinite(d)) {
                atomicAdd(bad, 1);
                d = 1.0;
            }
            col[0] = sqrt(d);
            Aj[0] = col[0];
        }
        __syncthreads();
        const double ljj = col[0];
        for (int i = 1 + tid; i <= m; i += kBandThreads) {
            const double v = Aj[i] / ljj;
            Aj[i] = v;
            col[i] = v;
        }
        __syncthreads();
        // a_{j+i, j+l} -= L_i L_l for 1 <= l <= i <= m (every pair a distinct entry)
        for (int l = 1; l <= m; l++) {
            const double cl = col[l];
            double *Al = A + (j + l) * (b + 1) - l;
            for (int i = l + tid; i <= m; i += kBandThreads) Al[i] -= col[i] * cl;
        }
        __syncthreads();
    }
}

// Narrow bands (b <= 31): one warp per wavenumber factors column by column
// with lane d holding L(j+d, j); the update of the next columns is lane-
// parallel, and __syncwarp orders it before the next column is read.
__global__ void __launch_bounds__(128) k_band_factor_warp(int64_t n, int b, int nK, double *__restrict__ B,
                                                           int32_t *__restrict__ bad) {
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= nK) return;
    double *A = B + (int64_t)w * n * (b + 1);
    for (int64_t j = 0; j < n; j++) {
        const int m = (int)(n - 1 - j < (int64_t)b ? n - 1 - j : (int64_t)b);
        double *Aj = A + j * (b + 1);
        double v = lane <= m ? Aj[lane] : 0.0;
        double d = __shfl_sync(0xffffffffu, v, 0);
        if (!(d > 0.0) || !isfinite(d)) {
            if (lane == 0) atomicAdd(bad, 1);
            d = 1.0;
        }
        const double ljj = sqrt(d);
        v = lane == 0 ? ljj : v / ljj;
        if (lane <= m) Aj[lane] = v;
        for (int l = 1; l <= m; l++) {
            const double cl = __shfl_sync(0xffffffffu, v, l);
            if (lane >= l && lane <= m) A[(j + l) * (b + 1) + (lane - l)] -= v * cl;
        }
        __syncwarp();
    }
}

// Narrow bands (b <= BW): one thread per right-hand side, the last BW
// solution values of its column in registers (pull form): forward
// y_j = (r_j - sum_{i=1..b} L(j, j-i) y_{j-i}) / L_jj with L(j, j-i) =
// B[(j-i)(b+1) + i], backward x_j = (y_j - sum_i L(j+i, j) x_{j+i}) / L_jj.
template <int BW>
__global__ void __launch_bounds__(128) k_band_solve_reg(int64_t n, int b, int nE, int64_t Rpad,
                                                         const double *__restrict__ B,
                                                         const int32_t *__restrict__ perm,
                                                         double *__restrict__ x) {
    const int k = blockIdx.y;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nE) return;
    const double *L = B + (int64_t)k * n * (b + 1);
    double *xc = x + (int64_t)k * nE + e;
    double win[BW];
#pragma unroll
    for (int i = 0; i < BW; i++) win[i] = 0.0;  // win[i] = y_{j-1-i}
    for (int64_t j = 0; j < n; j++) {
        const int64_t row = perm[j];
        double s0 = xc[row * Rpad], s1 = 0.0;
#pragma unroll
        for (int i = 0; i < BW; i++) {
            const int64_t c = j - 1 - i;  // column j-1-i holds L(j, c) at offset i+1
            if (i < b && c >= 0) {
                const double l = L[c * (b + 1) + i + 1];
                if (i & 1) s1 = fma(-l, win[i], s1);
                else s0 = fma(-l, win[i], s0);
            }
        }
        const double y = (s0 + s1) / L[j * (b + 1)];
        xc[row * Rpad] = y;
#pragma unroll
        for (int i = BW - 1; i > 0; i--) win[i] = win[i - 1];
        win[0] = y;
    }
#pragma unroll
    for (int i = 0; i < BW; i++) win[i] = 0.0;  // win[i] = x_{j+1+i}
    for (int64_t j = n - 1; j >= 0; j--) {
        const int64_t row = perm[j];
        const double *Lj = L + j * (b + 1);
        double s0 = xc[row * Rpad], s1 = 0.0;
#pragma unroll
        for (int i = 0; i < BW; i++) {
            if (i < b && j + 1 + i < n) {
                const double l = Lj[i + 1];
                if (i & 1) s1 = fma(-l, win[i], s1);
                else s0 = fma(-l, win[i], s0);
            }
        }
        const double xv = (s0 + s1) / Lj[0];
        xc[row * Rpad] = xv;
#pragma unroll
        for (int i = BW - 1; i > 0; i--) win[i] = win[i - 1];
        win[0] = xv;
    }
}

// one block per wavenumber, one thread per right-hand side of it: forward
// and backward substitution in place on x (node-major n x Rpad), rows
// visited in band order through perm
__global__ void __launch_bounds__(kBandThreads) k_band_solve(int64_t n, int b, int nE, int64_t Rpad,
                                                              const double *__restrict__ B,
                                                              const int32_t *__restrict__ perm,
                                                              double *__restrict__ x) {
    const int k = blockIdx.x;
    const double *L = B + (int64_t)k * n * (b + 1);
    for (int e = threadIdx.x; e < nE; e += blockDim.x) {
        double *xc = x + (int64_t)k * nE + e;
        for (int64_t j = 0; j < n; j++) {
            const double *Lj = L + j * (b + 1);
            const int m = (int)(n - 1 - j < (int64_t)b ? n - 1 - j : (int64_t)b);
            const double y = xc[(int64_t)perm[j] * Rpad] / Lj[0];
            xc[(int64_t)perm[j] * Rpad] = y;
            for (int i = 1; i <= m; i++) xc[(int64_t)perm[j + i] * Rpad] -= Lj[i] * y;
        }
        for (int64_t j = n - 1; j >= 0; j--) {
            const double *Lj = L + j * (b + 1);
            const int m = (int)(n - 1 - j < (int64_t)b ? n - 1 - j : (int64_t)b);
            double s = xc[(int64_t)perm[j] * Rpad];
            for (int i = 1; i <= m; i++) s -= Lj[i] * xc[(int64_t)perm[j + i] * Rpad];
            xc[(int64_t)perm[j] * Rpad] = s / Lj[0];
        }
    }
}

// bandwidth of the pattern under the order pos (old index -> new)
int bandwidth(int64_t n, const std::vector<int32_t> &rp, const std::vector<int32_t> &ci,
              const std::vector<int32_t> &pos) {
    int64_t bw = 0;
    for (int64_t i = 0; i < n; i++)
        for (int32_t q = rp[i]; q < rp[i + 1]; q++) bw = std::max<int64_t>(bw, std::abs((int64_t)pos[i] - pos[ci[q]]));
    return (int)std::min<int64_t>(bw, INT32_MAX);
}

// reverse Cuthill-McKee: breadth-first from a low-degree node of each
// component, neighbours by increasing degree, the order reversed
std::vector<int32_t> rcm_order(int64_t n, const std::vector<int32_t> &rp, const std::vector<int32_t> &ci) {
    std::vector<int32_t> order;
    order.reserve((size_t)n);
    std::vector<char> seen((size_t)n, 0);
    auto deg = [&](int64_t i) { return rp[i + 1] - rp[i]; };
    std::vector<int32_t> byDeg((size_t)n);
    for (int64_t i = 0; i < n; i++) byDeg[(size_t)i] = (int32_t)i;
    std::stable_sort(byDeg.begin(), byDeg.end(), [&](int32_t a, int32_t c) { return deg(a) < deg(c); });
    std::vector<int32_t> nb;
    for (int32_t start : byDeg) {
        if (seen[start]) continue;
        std::queue<int32_t> q;
        q.push(start);
        seen[start] = 1;
        while (!q.empty()) {
            const int32_t v = q.front();
            q.pop();
            order.push_back(v);
            nb.clear();
            for (int32_t p = rp[v]; p < rp[v + 1]; p++)
                if (!seen[ci[p]]) {
                    seen[ci[p]] = 1;
                    nb.push_back(ci[p]);
                }
            std::stable_sort(nb.begin(), nb.end(), [&](int32_t a, int32_t c) { return deg(a) < deg(c); });
            for (int32_t w : nb) q.push(w);
        }
    }
    std::reverse(order.begin(), order.end());
    return order;
}

void band_plan(Context &c) {
    MeshData &m = c.mesh;
    BandPlan &P = m.band;
    if (P.built) return;
    P.built = true;
    const int64_t n = m.n;
    std::vector<int32_t> ident((size_t)n);
    for (int64_t i = 0; i < n; i++) ident[(size_t)i] = (int32_t)i;
    const int b0 = bandwidth(n, m.rowptr, m.colidx, ident);
    std::vector<int32_t> perm = ident;
    int b = b0;
    if (b0 > 16) {
        std::vector<int32_t> rcm = rcm_order(n, m.rowptr, m.colidx), pos((size_t)n);
        for (int64_t i = 0; i < n; i++) pos[(size_t)rcm[(size_t)i]] = (int32_t)i;
        const int b1 = bandwidth(n, m.rowptr, m.colidx, pos);
        if (b1 < b0) {
            perm = rcm;
            b = b1;
        }
    }
    P.b = b;
    P.ok = b <= kMaxBand;
    if (!P.ok) return;
    P.perm = perm;
    P.pos.assign((size_t)n, 0);
    for (int64_t i = 0; i < n; i++) P.pos[(size_t)perm[(size_t)i]] = (int32_t)i;
    P.d_perm.upload(P.perm, c.stream);
    P.d_pos.upload(P.pos, c.stream);
}

}  // namespace

int band_solve(Context &c, cudaStream_t s) {
    MeshData &m = c.mesh;
    band_plan(c);
    const BandPlan &P = m.band;
    if (!P.ok)
        throw Error(ERTGB_BAD_INPUT, "the banded direct solve needs a matrix bandwidth of at most " +
                                         std::to_string(kMaxBand) + " (this matrix: " + std::to_string(P.b) +
                                         "); use an iterative preconditioner");
    const int64_t n = m.n, b = P.b;
    const size_t per = (size_t)n * (size_t)(b + 1);
    c.d_band.alloc(per * c.nK);
    ERTGB_CUDA(cudaMemsetAsync(c.d_band.p, 0, sizeof(double) * per * c.nK, s));
    k_band_fill<<<(unsigned)std::min<int64_t>(ceil_div(n * c.nK, kBandThreads), 4096), kBandThreads, 0, s>>>(n, (int)b, c.nK, m.nnz, m.d_rowptr.p, m.d_colidx.p,
                                                              P.d_pos.p, c.d_S.p, c.d_band.p);
    DBuf<int32_t> &bad = c.d_ic_bad;
    bad.alloc(1);
    bad.zero(s);
    if (b <= 31)
        k_band_factor_warp<<<(unsigned)ceil_div((int64_t)c.nK * 32, 128), 128, 0, s>>>(n, (int)b, c.nK, c.d_band.p,
                                                                                        bad.p);
    else
        k_band_factor<<<c.nK, kBandThreads, 0, s>>>(n, (int)b, c.d_band.p, bad.p);
    // the solution overwrites a copy of the right-hand sides (d_r keeps them)
    c.d_x.alloc((size_t)n * c.Rpad);
    ERTGB_CUDA(cudaMemcpyAsync(c.d_x.p, c.d_r.p, sizeof(double) * n * c.Rpad, cudaMemcpyDeviceToDevice, s));
    const dim3 sg((unsigned)ceil_div(c.nE, 32), (unsigned)c.nK);
    if (b <= 16)
        k_band_solve_reg<16><<<sg, 32, 0, s>>>(n, (int)b, c.nE, c.Rpad, c.d_band.p, P.d_perm.p, c.d_x.p);
    else if (b <= 32)
        k_band_solve_reg<32><<<sg, 32, 0, s>>>(n, (int)b, c.nE, c.Rpad, c.d_band.p, P.d_perm.p, c.d_x.p);
    else if (b <= 64)
        k_band_solve_reg<64><<<sg, 32, 0, s>>>(n, (int)b, c.nE, c.Rpad, c.d_band.p, P.d_perm.p, c.d_x.p);
    else
        k_band_solve<<<c.nK, std::min(kBandThreads, ((c.nE + 31) / 32) * 32), 0, s>>>(n, (int)b, c.nE, c.Rpad,
                                                                                      c.d_band.p, P.d_perm.p,
                                                                                      c.d_x.p);
    ERTGB_CUDA(cudaGetLastError());
    int32_t h = 0;
    ERTGB_CUDA(cudaMemcpyAsync(&h, bad.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    c.stats.iterations = 0;
    c.stats.max_rel_residual = 0.0;
    c.stats.n_rhs = (int32_t)c.R;
    c.stats.launches_response += 3;
    if (h) throw Error(ERTGB_NOT_CONVERGED, "banded Cholesky: " + std::to_string(h) + " pivots not positive");
    return ERTGB_OK;
}

}  // namespace ertgb
