// Mixed-precision multi-right-hand-side PCG: FP32 recurrence, FP64 accuracy.
//
// The CG recurrence (operator, Jacobi preconditioner, r, p, q and the
// solution increment y) runs in FP32, where GB300 has 55x the FP64 rate and
// the vector traffic halves.  Every kReliableEvery iterations a reliable
// update (Sleijpen & van der Vorst, "Reliable updated residuals in hybrid
// Bi-CG methods", Computing 56, 1996) folds the FP32 increment into the FP64
// solution, x += y, recomputes the true residual r = b - A x with the FP64
// matrix, and restarts the FP32 residual from it.  Convergence is decided
// only on that FP64 true residual (||r_t|| <= rtol ||b_t||), the same test
// as the FP64 solver, so the converged accuracy is unchanged.  Column dot
// products are accumulated in FP32 per thread and in FP64 across threads;
// the per-column scalars (alpha, beta, rho) stay FP64.
#include <algorithm>
#include <cmath>

#include "ertgb_internal.cuh"
#include "reduce.cuh"

namespace ertgb {

namespace {

constexpr int kRows = 8;            // warps per block (spmm) / rows per block (vector kernels)
constexpr int kGraphIters = 16;     // iterations per captured graph
constexpr int kReliableEvery = 4;   // graphs between reliable updates (64 iterations)
constexpr int kPartRows = 304;  // 2 row blocks per SM: few partial rows keep the column finishes short


__global__ void k_to_f32(int64_t n, const double *__restrict__ a, float *__restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// block reduction of two per-thread FP64 partials over threadIdx.y, written to
// part rows blockIdx.y (vector kernels: block (32, kRows), grid (Rpad/32, NB))
__device__ inline void block_partials2(double a, double b, double *part_a, double *part_b, int64_t Rpad, int64_t t) {
    __shared__ double sa[kRows][32], sb[kRows][32];
    sa[threadIdx.y][threadIdx.x] = a;
    sb[threadIdx.y][threadIdx.x] = b;
    __syncthreads();
    if (threadIdx.y == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < kRows; w++) {
            s1 += sa[w][threadIdx.x];
            s2 += sb[w][threadIdx.x];
        }
        part_a[(int64_t)blockIdx.y * Rpad + t] = s1;
        part_b[(int64_t)blockIdx.y * Rpad + t] = s2;
    }
}

__global__ void k_m_init(int64_t n, int nE, int64_t R, int64_t Rpad, const float *__restrict__ dinv,
                         const double *__restrict__ b, float *__restrict__ r, float *__restrict__ p,
                         float *__restrict__ y, double *__restrict__ part_a, double *__restrict__ part_b) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const int64_t ki = t < R ? t / nE : 0;
    const float *dk = dinv + ki * n;
    float a = 0.f;
    double bb = 0.0;
#pragma unroll 4
    for (int64_t row = (int64_t)blockIdx.y * kRows + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRows) {
        const int64_t i = row * Rpad + t;
        const double bv = b[i];
        const float rv = (float)bv;
        const float z = t < R ? rv * dk[row] : 0.f;
        r[i] = rv;
        p[i] = z;
        y[i] = 0.f;
        a = fmaf(rv, z, a);
        bb = fma(bv, bv, bb);
    }
    block_partials2((double)a, bb, part_a, part_b, Rpad, t);
}

template <int CH>
__global__ void __launch_bounds__(256) k_spmm32_dot(int64_t n, int64_t nnz, int nE, int nK, int64_t Rpad,
                                                    const int32_t *__restrict__ rowptr,
                                                    const int32_t *__restrict__ colidx,
                                                    const float *__restrict__ vals, const float *__restrict__ p,
                                                    float *__restrict__ q, double *__restrict__ part) {
    __shared__ double red[kRows][32 * CH];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t t0 = (int64_t)blockIdx.y * 32 * CH + lane;
    int64_t kofs[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) kofs[j] = min((t0 + 32 * j) / nE, (int64_t)nK - 1) * nnz;
    float dot[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) dot[j] = 0.f;
    for (int64_t row = (int64_t)blockIdx.x * kRows + wid; row < n; row += (int64_t)gridDim.x * kRows) {
        float acc[CH];
#pragma unroll
        for (int j = 0; j < CH; j++) acc[j] = 0.f;
        const int32_t s1 = rowptr[row + 1];
        for (int32_t s = rowptr[row]; s < s1; s++) {
            const int64_t col = colidx[s];
            const float *pc = p + col * Rpad + t0;
#pragma unroll
            for (int j = 0; j < CH; j++) acc[j] = fmaf(vals[kofs[j] + s], pc[32 * j], acc[j]);
        }
        float *qr = q + row * Rpad + t0;
        const float *pr = p + row * Rpad + t0;
#pragma unroll
        for (int j = 0; j < CH; j++) {
            qr[32 * j] = acc[j];
            dot[j] = fmaf(pr[32 * j], acc[j], dot[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < CH; j++) red[wid][lane + 32 * j] = (double)dot[j];
    __syncthreads();
    for (int c = threadIdx.x; c < 32 * CH; c += blockDim.x) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kRows; w++) s += red[w][c];
        part[(int64_t)blockIdx.x * Rpad + (int64_t)blockIdx.y * 32 * CH + c] = s;
    }
}

// Single-matrix variant (nK = 1): an 8-lane group per matrix row, every lane
// gathering CH float4 of the 32*CH columns of the chunk (coalesced 128-byte
// segments per group), so a warp keeps four rows and, with the unrolled
// nonzero loop, many gathers of p in flight.  Every block owns a contiguous
// range of rows (neighbour rows share their gathers of p through L1).  The
// column dots are summed per lane in FP32 and across the block's groups in
// FP64, in a fixed order.
// DOT: 0 = column dots p . q (the PCG operator), 1 = none, 2 = w . q.
constexpr int kQThreads = 256;
constexpr int kQGroups = kQThreads / 8;
constexpr int kQTileRows = 128;  // rows per tile of the FP32 operator (a multiple of kQGroups)

template <int CH, int DOT>
__global__ void __launch_bounds__(kQThreads, 2) k_spmm32_q(int64_t n, int64_t Rpad, const int32_t *__restrict__ rowptr,
                                                           const int32_t *__restrict__ colidx,
                                                           const float *__restrict__ vals, const float *__restrict__ p,
                                                           float *__restrict__ q, const float *__restrict__ w,
                                                           double *__restrict__ part) {
    __shared__ float red[DOT == 1 ? 1 : kQGroups][DOT == 1 ? 1 : 32 * CH + 1];
    const int l8 = threadIdx.x & 7, g = threadIdx.x >> 3;
    const int64_t t0 = (int64_t)blockIdx.y * 32 * CH + l8 * 4;
    float4 dot[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) dot[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    // tiles of kQTileRows consecutive rows in grid-stride order: the rows in
    // flight at a time form one window of consecutive rows, so the rows of p
    // that neighbouring matrix rows share stay in L2 when p exceeds it
    const int64_t ntile = (n + kQTileRows - 1) / kQTileRows;
    for (int64_t tile = blockIdx.x; tile < ntile; tile += gridDim.x)
    for (int64_t row = tile * kQTileRows + g, r_end = min(n, (tile + 1) * kQTileRows); row < r_end;
         row += kQGroups) {
        float4 acc[CH];
#pragma unroll
        for (int j = 0; j < CH; j++) acc[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        const int32_t s1 = rowptr[row + 1];
#pragma unroll 4
        for (int32_t s = rowptr[row]; s < s1; s++) {
            const int64_t col = colidx[s];
            const float v = vals[s];
            const float4 *pc = reinterpret_cast<const float4 *>(p + col * Rpad + t0);
#pragma unroll
            for (int j = 0; j < CH; j++) {
                const float4 x = __ldg(pc + 8 * j);
                acc[j].x = fmaf(v, x.x, acc[j].x);
                acc[j].y = fmaf(v, x.y, acc[j].y);
                acc[j].z = fmaf(v, x.z, acc[j].z);
                acc[j].w = fmaf(v, x.w, acc[j].w);
            }
        }
        float4 *qr = reinterpret_cast<float4 *>(q + row * Rpad + t0);
#pragma unroll
        for (int j = 0; j < CH; j++) qr[8 * j] = acc[j];
        if (DOT != 1) {
            const float4 *dr = reinterpret_cast<const float4 *>((DOT == 2 ? w : p) + row * Rpad + t0);
#pragma unroll
            for (int j = 0; j < CH; j++) {
                const float4 d = dr[8 * j];
                dot[j].x = fmaf(d.x, acc[j].x, dot[j].x);
                dot[j].y = fmaf(d.y, acc[j].y, dot[j].y);
                dot[j].z = fmaf(d.z, acc[j].z, dot[j].z);
                dot[j].w = fmaf(d.w, acc[j].w, dot[j].w);
            }
        }
    }
    if (DOT == 1) return;
#pragma unroll
    for (int j = 0; j < CH; j++) {
        const int c = 32 * j + l8 * 4;
        red[g][c] = dot[j].x;
        red[g][c + 1] = dot[j].y;
        red[g][c + 2] = dot[j].z;
        red[g][c + 3] = dot[j].w;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < 32 * CH; c += kQThreads) {
        double s = 0.0;
#pragma unroll
        for (int gg = 0; gg < kQGroups; gg++) s += (double)red[gg][c];
        part[(int64_t)blockIdx.x * Rpad + (int64_t)blockIdx.y * 32 * CH + c] = s;
    }
}

// Generic FP32 CSR product y = B x for the FSAI factors (nK value arrays of
// stride nnzB; warp per row, lanes over columns); with DOT the column
// partials of w . y are written to part.
template <int CH, bool DOT>
__global__ void __launch_bounds__(256) k_spmm32_gen(int64_t n, int64_t nnzB, int nE, int nK, int64_t Rpad,
                                                    const int32_t *__restrict__ rowptr,
                                                    const int32_t *__restrict__ colidx,
                                                    const float *__restrict__ vals, const float *__restrict__ x,
                                                    float *__restrict__ y, const float *__restrict__ w,
                                                    double *__restrict__ part) {
    __shared__ double red[kRows][32 * CH];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t t0 = (int64_t)blockIdx.y * 32 * CH + lane;
    int64_t kofs[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) kofs[j] = min((t0 + 32 * j) / nE, (int64_t)nK - 1) * nnzB;
    float dot[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) dot[j] = 0.f;
    const int64_t per_block = (n + gridDim.x - 1) / gridDim.x;
    const int64_t r_begin = (int64_t)blockIdx.x * per_block, r_end = min(n, r_begin + per_block);
    for (int64_t row = r_begin + wid; row < r_end; row += kRows) {
        float acc[CH];
#pragma unroll
        for (int j = 0; j < CH; j++) acc[j] = 0.f;
        const int32_t s1 = rowptr[row + 1];
#pragma unroll 2
        for (int32_t s = rowptr[row]; s < s1; s++) {
            const int64_t col = colidx[s];
            const float *xc = x + col * Rpad + t0;
#pragma unroll
            for (int j = 0; j < CH; j++) acc[j] = fmaf(vals[kofs[j] + s], xc[32 * j], acc[j]);
        }
#pragma unroll
        for (int j = 0; j < CH; j++) {
            y[row * Rpad + t0 + 32 * j] = acc[j];
            if (DOT) dot[j] = fmaf(w[row * Rpad + t0 + 32 * j], acc[j], dot[j]);
        }
    }
    if (!DOT) return;
#pragma unroll
    for (int j = 0; j < CH; j++) red[wid][lane + 32 * j] = (double)dot[j];
    __syncthreads();
    for (int c = threadIdx.x; c < 32 * CH; c += blockDim.x) {
        double s = 0.0;
#pragma unroll
        for (int w2 = 0; w2 < kRows; w2++) s += red[w2][c];
        part[(int64_t)blockIdx.x * Rpad + (int64_t)blockIdx.y * 32 * CH + c] = s;
    }
}

// FSAI iteration: y += alpha p, r -= alpha q (the dots follow from z = G^T G r)
// FSAI / learned iteration, first half: r -= alpha q
__global__ void k_m_update_r(int64_t n, int64_t Rpad, const double *__restrict__ col,
                             const int32_t *__restrict__ active, float *__restrict__ r, const float *__restrict__ q) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (!active[t]) return;
    const float alpha = (float)col[ALPHA * Rpad + t];
#pragma unroll 4
    for (int64_t row = (int64_t)blockIdx.y * kRows + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRows) {
        const int64_t i = row * Rpad + t;
        r[i] = fmaf(-alpha, q[i], r[i]);
    }
}

// second half, after beta: y += alpha p with the p of this iteration, then
// p = z + beta p (one pass over p for both)
__global__ void k_m_update_pzy(int64_t n, int64_t Rpad, const double *__restrict__ col,
                               const int32_t *__restrict__ active, const float *__restrict__ z, float *__restrict__ p,
                               float *__restrict__ y) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (!active[t]) return;
    const float alpha = (float)col[ALPHA * Rpad + t];
    const float beta = (float)col[BETA * Rpad + t];
#pragma unroll 4
    for (int64_t row = (int64_t)blockIdx.y * kRows + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRows) {
        const int64_t i = row * Rpad + t;
        const float pv = p[i];
        y[i] = fmaf(alpha, pv, y[i]);
        p[i] = fmaf(beta, pv, z[i]);
    }
}

__global__ void k_m_update_xr(int64_t n, int nE, int64_t R, int64_t Rpad, const float *__restrict__ dinv,
                              const double *__restrict__ col, const int32_t *__restrict__ active,
                              float *__restrict__ y, float *__restrict__ r, const float *__restrict__ p,
                              const float *__restrict__ q, double *__restrict__ part_a, double *__restrict__ part_b) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const bool act = active[t] != 0;
    const float alpha = (float)col[ALPHA * Rpad + t];
    const int64_t ki = t < R ? t / nE : 0;
    const float *dk = dinv + ki * n;
    float a = 0.f, b = 0.f;
    if (act) {
    #pragma unroll 4
    for (int64_t row = (int64_t)blockIdx.y * kRows + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRows) {
            const int64_t i = row * Rpad + t;
            y[i] = fmaf(alpha, p[i], y[i]);
            const float rv = fmaf(-alpha, q[i], r[i]);
            r[i] = rv;
            a = fmaf(rv, rv * dk[row], a);
            b = fmaf(rv, rv, b);
        }
    }
    block_partials2((double)a, (double)b, part_a, part_b, Rpad, t);
}

// alpha = rho / (p . q) per active column
__global__ void k_m_finish_alpha_w(int64_t Rpad, int NB, const double *__restrict__ part, double *__restrict__ col,
                                   const int32_t *__restrict__ active, int32_t *__restrict__ nactive) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *nactive = 0;
    const int64_t t = (int64_t)blockIdx.x * kFinWarps + (threadIdx.x >> 5);
    if (t >= Rpad) return;  // whole warps
    const double pq = warp_col_sum(part, NB, Rpad, t);
    if ((threadIdx.x & 31) != 0 || !active[t]) return;
    col[PQ * Rpad + t] = pq;
    col[ALPHA * Rpad + t] = (pq != 0.0) ? col[RHO * Rpad + t] / pq : 0.0;
}

// recursive beta; convergence is left to the reliable updates
__global__ void k_m_finish_beta_w(int64_t Rpad, int NB, const double *__restrict__ part_a, double *__restrict__ col,
                                  const int32_t *__restrict__ active, int32_t *__restrict__ iters) {
    const int64_t t = (int64_t)blockIdx.x * kFinWarps + (threadIdx.x >> 5);
    if (t >= Rpad) return;
    const double rz = warp_col_sum(part_a, NB, Rpad, t);
    if ((threadIdx.x & 31) != 0) return;
    if (!active[t]) {
        col[BETA * Rpad + t] = 0.0;
        return;
    }
    iters[t] += 1;
    const double rho = col[RHO * Rpad + t];
    col[BETA * Rpad + t] = (rho != 0.0 && rz == rz) ? rz / rho : 0.0;
    col[RHO * Rpad + t] = rz;
}

__global__ void k_m_update_p(int64_t n, int nE, int64_t R, int64_t Rpad, const float *__restrict__ dinv,
                             const double *__restrict__ col, const int32_t *__restrict__ active,
                             const float *__restrict__ r, float *__restrict__ p) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (!active[t]) return;
    const float beta = (float)col[BETA * Rpad + t];
    const int64_t ki = t < R ? t / nE : 0;
    const float *dk = dinv + ki * n;
#pragma unroll 4
    for (int64_t row = (int64_t)blockIdx.y * kRows + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRows) {
        const int64_t i = row * Rpad + t;
        p[i] = fmaf(beta, p[i], r[i] * dk[row]);
    }
}

// reliable update, part 1: x += y, y = 0 on active columns
__global__ void k_m_accum(int64_t n, int64_t Rpad, const int32_t *__restrict__ active, double *__restrict__ x,
                          float *__restrict__ y, int32_t *__restrict__ nactive) {
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) *nactive = 0;
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (!active[t]) return;
#pragma unroll 4
    for (int64_t row = (int64_t)blockIdx.y * kRows + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRows) {
        const int64_t i = row * Rpad + t;
        x[i] += (double)y[i];
        y[i] = 0.f;
    }
}

// reliable update, part 2: true residual r = b - A x in FP64 (warp per row,
// lanes over columns), restart r32 from it, partials of r32.z32 and ||r||^2
template <int CH>
__global__ void __launch_bounds__(256) k_m_residual(int64_t n, int64_t nnz, int nE, int nK, int64_t R, int64_t Rpad,
                                                    const int32_t *__restrict__ rowptr,
                                                    const int32_t *__restrict__ colidx,
                                                    const double *__restrict__ vals, const double *__restrict__ x,
                                                    const double *__restrict__ b, const float *__restrict__ dinv,
                                                    const int32_t *__restrict__ active, float *__restrict__ r32,
                                                    double *__restrict__ part_a, double *__restrict__ part_b) {
    __shared__ double ra[kRows][32 * CH], rb[kRows][32 * CH];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t t0 = (int64_t)blockIdx.y * 32 * CH + lane;
    int64_t kofs[CH], kdi[CH];
    bool act[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) {
        const int64_t t = t0 + 32 * j;
        const int64_t ki = min(t / nE, (int64_t)nK - 1);
        kofs[j] = ki * nnz;
        kdi[j] = ki * n;
        act[j] = active[t] != 0;
    }
    double sa[CH], sb[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) sa[j] = sb[j] = 0.0;
    for (int64_t row = (int64_t)blockIdx.x * kRows + wid; row < n; row += (int64_t)gridDim.x * kRows) {
        double acc[CH];
#pragma unroll
        for (int j = 0; j < CH; j++) acc[j] = 0.0;
        const int32_t s1 = rowptr[row + 1];
        for (int32_t s = rowptr[row]; s < s1; s++) {
            const int64_t col = colidx[s];
            const double *xc = x + col * Rpad + t0;
#pragma unroll
            for (int j = 0; j < CH; j++)
                if (act[j]) acc[j] = fma(vals[kofs[j] + s], xc[32 * j], acc[j]);
        }
#pragma unroll
        for (int j = 0; j < CH; j++) {
            if (!act[j]) continue;
            const int64_t i = row * Rpad + t0 + 32 * j;
            const double rv = b[i] - acc[j];
            const float r = (float)rv;
            r32[i] = r;
            sa[j] += (double)(r * (r * dinv[kdi[j] + row]));
            sb[j] = fma(rv, rv, sb[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < CH; j++) {
        ra[wid][lane + 32 * j] = sa[j];
        rb[wid][lane + 32 * j] = sb[j];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < 32 * CH; c += blockDim.x) {
        double s1 = 0.0, s2 = 0.0;
#pragma unroll
        for (int w = 0; w < kRows; w++) {
            s1 += ra[w][c];
            s2 += rb[w][c];
        }
        part_a[(int64_t)blockIdx.x * Rpad + (int64_t)blockIdx.y * 32 * CH + c] = s1;
        part_b[(int64_t)blockIdx.x * Rpad + (int64_t)blockIdx.y * 32 * CH + c] = s2;
    }
}

// reliable update, part 3: FP64 convergence test on the true residual, rho
// of the restarted residual, and stall detection.  A column whose best true
// residual has not improved by 10 % over four reliable-update intervals
// (256 iterations), or whose FP32 recurrence diverged (residual above twice
// the right-hand side, or not finite), stops here and is finished by the
// FP64 solver: nearly singular systems such as the smallest 2.5-D
// wavenumbers are beyond FP32 (their FP32 matrix can lose definiteness).
// stalled[t] = 1: warm start from the FP64 solution; 2: restart from zero.
__global__ void k_m_finish_ru(int64_t Rpad, int NB, double rtol2, const double *__restrict__ part_a,
                              const double *__restrict__ part_b, double *__restrict__ col, ColState cs) {
    __shared__ double ra[32][33], rb[32][33];
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const double rz = col_sum(part_a, NB, Rpad, t, ra);
    const double rr = col_sum(part_b, NB, Rpad, t, rb);
    if (threadIdx.y != 0 || !cs.active[t]) return;
    const double bb = col[BNORM2 * Rpad + t];
    col[RNORM2 * Rpad + t] = rr;
    col[RHO * Rpad + t] = rz;
    if (rr <= rtol2 * bb) {
        cs.active[t] = 0;
        return;
    }
    if (!(rr <= 4.0 * bb) || !(rz == rz)) {  // diverged or not finite
        cs.active[t] = 0;
        cs.stalled[t] = 2;
        atomicAdd(cs.nstalled, 1);
        return;
    }
    const double best = col[RPREV * Rpad + t];
    double stalls = col[STALLS * Rpad + t];
    if (rr < 0.81 * best) {
        col[RPREV * Rpad + t] = rr;
        stalls = 0.0;
    } else {
        stalls += 1.0;
    }
    col[STALLS * Rpad + t] = stalls;
    if (stalls >= 4.0) {
        cs.active[t] = 0;
        cs.stalled[t] = 1;
        atomicAdd(cs.nstalled, 1);
        return;
    }
    atomicAdd(cs.nactive, 1);
}

// columns of wavenumbers that stalled in FP32 in the previous response go
// straight to the FP64 solver (stalled = 2: from zero)
__global__ void k_m_pre_fp64(int64_t Rpad, const int32_t *__restrict__ pre, ColState cs) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Rpad || !pre[t] || !cs.active[t]) return;
    cs.active[t] = 0;
    cs.stalled[t] = 2;
    atomicSub(cs.nactive, 1);
    atomicAdd(cs.nstalled, 1);
}

int choose_ch(int64_t Rpad) {
    const int64_t w = Rpad / 32;
    for (int ch : {4, 3, 2})
        if (w % ch == 0) return ch;
    return 1;
}

template <template <int> class F, typename... A> void dispatch_ch(int ch, A &&...args) {
    switch (ch) {
        case 4: F<4>::go(args...); break;
        case 3: F<3>::go(args...); break;
        case 2: F<2>::go(args...); break;
        default: F<1>::go(args...); break;
    }
}

template <int CH> struct SpmmL {
    static void go(dim3 g, cudaStream_t s, int64_t n, int64_t nnz, int nE, int nK, int64_t Rpad, const int32_t *rp,
                   const int32_t *ci, const float *v, const float *p, float *q, double *part) {
        if (nK == 1) k_spmm32_q<CH, 0><<<g, kQThreads, 0, s>>>(n, Rpad, rp, ci, v, p, q, nullptr, part);
        else k_spmm32_dot<CH><<<g, 256, 0, s>>>(n, nnz, nE, nK, Rpad, rp, ci, v, p, q, part);
    }
};

template <int CH> struct GenL {
    static void go(dim3 g, cudaStream_t s, int64_t n, int64_t nnzB, int nE, int nK, int64_t Rpad, const int32_t *rp,
                   const int32_t *ci, const float *v, const float *x, float *y, const float *w, double *part) {
        if (nK == 1) {
            if (w) k_spmm32_q<CH, 2><<<g, kQThreads, 0, s>>>(n, Rpad, rp, ci, v, x, y, w, part);
            else k_spmm32_q<CH, 1><<<g, kQThreads, 0, s>>>(n, Rpad, rp, ci, v, x, y, w, part);
        } else if (w) {
            k_spmm32_gen<CH, true><<<g, 256, 0, s>>>(n, nnzB, nE, nK, Rpad, rp, ci, v, x, y, w, part);
        } else {
            k_spmm32_gen<CH, false><<<g, 256, 0, s>>>(n, nnzB, nE, nK, Rpad, rp, ci, v, x, y, w, part);
        }
    }
};

template <int CH> struct ResidL {
    static void go(dim3 g, cudaStream_t s, int64_t n, int64_t nnz, int nE, int nK, int64_t R, int64_t Rpad,
                   const int32_t *rp, const int32_t *ci, const double *v, const double *x, const double *b,
                   const float *dinv, const int32_t *active, float *r32, double *pa, double *pb) {
        k_m_residual<CH><<<g, 256, 0, s>>>(n, nnz, nE, nK, R, Rpad, rp, ci, v, x, b, dinv, active, r32, pa, pb);
    }
};

}  // namespace

int pcg_solve_mixed(Context &c, cudaStream_t s) {
    MeshData &m = c.mesh;
    const int64_t n = m.n, Rpad = c.Rpad, R = c.R;
    const int NB = (int)std::min<int64_t>(ceil_div(n, kRows), kPartRows);
    const int ch = choose_ch(Rpad);
    const int nchunk = (int)(Rpad / (32 * ch));
    c.d_x.alloc((size_t)n * Rpad);
    c.d_S32.alloc((size_t)c.nK * m.nnz);
    c.d_dinv32.alloc((size_t)c.nK * n);
    c.d_r32.alloc((size_t)n * Rpad);
    c.d_p32.alloc((size_t)n * Rpad);
    c.d_q32.alloc((size_t)n * Rpad);
    c.d_y32.alloc((size_t)n * Rpad);
    c.d_part.alloc((size_t)NB * Rpad * 3);
    c.d_col.alloc((size_t)NCOL * Rpad);
    c.d_active.alloc(ColState::size(Rpad));
    double *part_a = c.d_part.p, *part_b = c.d_part.p + (size_t)NB * Rpad, *part_c = c.d_part.p + 2 * (size_t)NB * Rpad;
    ColState cs(c.d_active.p, Rpad);
    int32_t *active = cs.active, *iters = cs.iters, *nactive = cs.nactive;
    const double *b = c.d_r.p;  // the right-hand sides (FP64), kept for the true residual
    const bool fsai = c.precond != ERTGB_PRECOND_JACOBI;  // FSAI or learned: the same G^T G application
    const int64_t nL = (int64_t)m.Lcolidx.size();
    if (fsai) {
        if (c.precond == ERTGB_PRECOND_FSAI)
            fsai_setup(c, s);
        else
            lp_setup(c, s);
        c.d_t32.alloc((size_t)n * Rpad);
        c.d_z32.alloc((size_t)n * Rpad);
    }
    // z = G^T (G r) with the column partials of r . z into pz
    auto apply_fsai = [&](double *pz) {
        dispatch_ch<GenL>(ch, dim3((unsigned)NB, (unsigned)nchunk), s, n, nL, c.nE, c.nK, Rpad, m.d_Lrowptr.p,
                          m.d_Lcolidx.p, c.d_G32.p, c.d_r32.p, c.d_t32.p, (const float *)nullptr, (double *)nullptr);
        dispatch_ch<GenL>(ch, dim3((unsigned)NB, (unsigned)nchunk), s, n, nL, c.nE, c.nK, Rpad, m.d_Urowptr.p,
                          m.d_Ucolidx.p, c.d_GT32.p, c.d_t32.p, c.d_z32.p, (const float *)c.d_r32.p, pz);
    };
    ERTGB_CUDA(cudaMemsetAsync(c.d_x.p, 0, sizeof(double) * n * Rpad, s));
    ERTGB_CUDA(cudaMemsetAsync(cs.stalled, 0, sizeof(int32_t) * (Rpad + 2), s));  // stalled flags + counters
    k_to_f32<<<(unsigned)std::min<int64_t>(ceil_div((int64_t)c.nK * m.nnz, 256), 65535), 256, 0, s>>>(
        (int64_t)c.nK * m.nnz, c.d_S.p, c.d_S32.p);
    k_to_f32<<<(unsigned)std::min<int64_t>(ceil_div((int64_t)c.nK * n, 256), 65535), 256, 0, s>>>(
        (int64_t)c.nK * n, c.d_dinv.p, c.d_dinv32.p);
    const dim3 vb(32, kRows), vg((unsigned)(Rpad / 32), (unsigned)NB);
    // vector updates without column partials (FSAI / learned form) are free to use more row blocks
    const dim3 vgu((unsigned)(Rpad / 32), (unsigned)std::min<int64_t>(ceil_div(n, kRows), 4 * kPartRows));
    const dim3 sg((unsigned)NB, (unsigned)nchunk);
    const dim3 fb(32, 32), fg((unsigned)(Rpad / 32));
    const unsigned fwg = (unsigned)ceil_div(Rpad, kFinWarps);
    const double rtol2 = c.rtol * c.rtol;
    k_m_init<<<vg, vb, 0, s>>>(n, c.nE, R, Rpad, c.d_dinv32.p, b, c.d_r32.p, c.d_p32.p, c.d_y32.p, part_a, part_b);
    if (fsai) {
        apply_fsai(part_a);
        ERTGB_CUDA(cudaMemcpyAsync(c.d_p32.p, c.d_z32.p, sizeof(float) * n * Rpad, cudaMemcpyDeviceToDevice, s));
        c.stats.launches_response += 2;
    }
    pcg_finish_init(fg, fb, s, Rpad, R, NB, part_a, part_b, c.d_col.p, active, iters, nactive,
                    c.d_pnorm2.n >= (size_t)Rpad ? c.d_pnorm2.p : nullptr);
    ERTGB_CUDA(cudaGetLastError());
    c.stats.launches_response += 5;
    if ((int)c.fp64_k.size() == c.nK) {
        std::vector<int32_t> pre((size_t)Rpad, 0);
        int32_t n_pre = 0;
        for (int64_t t = 0; t < R; t++)
            if (c.fp64_k[(size_t)(t / c.nE)]) {
                pre[(size_t)t] = 1;
                n_pre++;
            }
        if (n_pre) {
            c.d_pre.upload(pre, s);
            k_m_pre_fp64<<<(unsigned)ceil_div(Rpad, 256), 256, 0, s>>>(Rpad, c.d_pre.p, cs);
            ERTGB_CUDA(cudaGetLastError());
            c.stats.launches_response += 1;
        }
    }

    cudaGraph_t g_it = nullptr, g_ru = nullptr;
    cudaGraphExec_t e_it = nullptr, e_ru = nullptr;
    auto cleanup = [&] {
        if (e_it) cudaGraphExecDestroy(e_it);
        if (g_it) cudaGraphDestroy(g_it);
        if (e_ru) cudaGraphExecDestroy(e_ru);
        if (g_ru) cudaGraphDestroy(g_ru);
    };
    int status = ERTGB_OK;
    int iterations = 0;
    try {
        ERTGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int it = 0; it < kGraphIters; it++) {
            dispatch_ch<SpmmL>(ch, sg, s, n, m.nnz, c.nE, c.nK, Rpad, m.d_rowptr.p, m.d_colidx.p, c.d_S32.p, c.d_p32.p,
                               c.d_q32.p, part_c);
            k_m_finish_alpha_w<<<fwg, 32 * kFinWarps, 0, s>>>(Rpad, NB, part_c, c.d_col.p, active, nactive);
            if (fsai) {
                k_m_update_r<<<vgu, vb, 0, s>>>(n, Rpad, c.d_col.p, active, c.d_r32.p, c.d_q32.p);
                apply_fsai(part_a);
                k_m_finish_beta_w<<<fwg, 32 * kFinWarps, 0, s>>>(Rpad, NB, part_a, c.d_col.p, active, iters);
                k_m_update_pzy<<<vgu, vb, 0, s>>>(n, Rpad, c.d_col.p, active, c.d_z32.p, c.d_p32.p, c.d_y32.p);
            } else {
                k_m_update_xr<<<vg, vb, 0, s>>>(n, c.nE, R, Rpad, c.d_dinv32.p, c.d_col.p, active, c.d_y32.p,
                                                c.d_r32.p, c.d_p32.p, c.d_q32.p, part_a, part_b);
                k_m_finish_beta_w<<<fwg, 32 * kFinWarps, 0, s>>>(Rpad, NB, part_a, c.d_col.p, active, iters);
                k_m_update_p<<<vg, vb, 0, s>>>(n, c.nE, R, Rpad, c.d_dinv32.p, c.d_col.p, active, c.d_r32.p,
                                               c.d_p32.p);
            }
        }
        ERTGB_CUDA(cudaStreamEndCapture(s, &g_it));
        ERTGB_CUDA(cudaGraphInstantiate(&e_it, g_it, 0));
        ERTGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        k_m_accum<<<vg, vb, 0, s>>>(n, Rpad, active, c.d_x.p, c.d_y32.p, nactive);
        dispatch_ch<ResidL>(ch, sg, s, n, m.nnz, c.nE, c.nK, R, Rpad, m.d_rowptr.p, m.d_colidx.p, c.d_S.p, c.d_x.p,
                            b, c.d_dinv32.p, active, c.d_r32.p, part_a, part_b);
        if (fsai) apply_fsai(part_a);
        k_m_finish_ru<<<fg, fb, 0, s>>>(Rpad, NB, rtol2, part_a, part_b, c.d_col.p, cs);
        ERTGB_CUDA(cudaStreamEndCapture(s, &g_ru));
        ERTGB_CUDA(cudaGraphInstantiate(&e_ru, g_ru, 0));

        int32_t h_active = 0;
        ERTGB_CUDA(cudaMemcpyAsync(&h_active, nactive, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        ERTGB_CUDA(cudaStreamSynchronize(s));
        while (h_active > 0) {
            if (iterations >= c.max_iter) {
                status = ERTGB_NOT_CONVERGED;
                break;
            }
            for (int u = 0; u < kReliableEvery; u++) ERTGB_CUDA(cudaGraphLaunch(e_it, s));
            iterations += kReliableEvery * kGraphIters;
            ERTGB_CUDA(cudaGraphLaunch(e_ru, s));
            c.stats.launches_response += (fsai ? 6 : 5) * kGraphIters * kReliableEvery + (fsai ? 5 : 3);
            ERTGB_CUDA(cudaMemcpyAsync(&h_active, nactive, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            ERTGB_CUDA(cudaStreamSynchronize(s));
        }
    } catch (...) {
        cudaStreamEndCapture(s, &g_it);
        cleanup();
        throw;
    }
    cleanup();
    int32_t h_stalled = 0;
    ERTGB_CUDA(cudaMemcpyAsync(&h_stalled, cs.nstalled, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    c.stats.stalled_columns = h_stalled;
    if (status == ERTGB_OK) {  // wavenumbers with at least half of their columns stalled start in FP64 next time
        std::vector<int32_t> st((size_t)Rpad);
        ERTGB_CUDA(cudaMemcpyAsync(st.data(), cs.stalled, sizeof(int32_t) * Rpad, cudaMemcpyDeviceToHost, s));
        ERTGB_CUDA(cudaStreamSynchronize(s));
        c.fp64_k.assign((size_t)c.nK, 0);
        for (int k = 0; k < c.nK; k++) {
            int cnt = 0;
            for (int e = 0; e < c.nE; e++) cnt += st[(size_t)k * c.nE + e] != 0;
            c.fp64_k[(size_t)k] = 2 * cnt >= c.nE ? 1 : 0;
        }
    }
    if (status == ERTGB_OK && h_stalled > 0) {
        // FP64 PCG on the stalled columns, warm-started from their FP64 solution
        c.stats.iterations = 0;
        return pcg_solve(c, s, cs.stalled);
    }
    std::vector<int32_t> it_h(Rpad);
    std::vector<double> rn(Rpad), bn(Rpad);
    ERTGB_CUDA(cudaMemcpyAsync(it_h.data(), iters, sizeof(int32_t) * Rpad, cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaMemcpyAsync(rn.data(), c.d_col.p + RNORM2 * Rpad, sizeof(double) * Rpad, cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaMemcpyAsync(bn.data(), c.d_col.p + BNORM2 * Rpad, sizeof(double) * Rpad, cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    int maxit = 0;
    double maxres = 0.0;
    bool finite = true;
    for (int64_t t = 0; t < R; t++) {
        maxit = std::max(maxit, it_h[t]);
        if (bn[t] > 0) {
            const double rel = std::sqrt(rn[t] / bn[t]);
            if (!std::isfinite(rel)) finite = false;
            else maxres = std::max(maxres, rel);
        }
    }
    if (!finite) {
        status = ERTGB_NOT_CONVERGED;
        maxres = NAN;
    }
    c.stats.iterations = maxit;
    c.stats.n_rhs = (int32_t)R;
    c.stats.max_rel_residual = maxres;
    return status;
}

void profile_spmm32(Context &c, int reps, double *ms, double *bytes, double *flops) {
    MeshData &m = c.mesh;
    const int64_t n = m.n, Rpad = c.Rpad;
    const int NB = (int)std::min<int64_t>(ceil_div(n, kRows), kPartRows);
    const int ch = choose_ch(Rpad);
    const dim3 sg((unsigned)NB, (unsigned)(Rpad / (32 * ch)));
    if (c.d_q32.n < (size_t)n * Rpad || c.d_S32.n < (size_t)c.nK * m.nnz)
        throw Error(ERTGB_STATE, "profile needs a completed mixed-precision response");
    if (c.d_part.n < (size_t)NB * Rpad * 3) c.d_part.alloc((size_t)NB * Rpad * 3);
    cudaStream_t s = c.stream;
    double *part_c = c.d_part.p + 2 * (size_t)NB * Rpad;
    auto go = [&] {
        dispatch_ch<SpmmL>(ch, sg, s, n, m.nnz, c.nE, c.nK, Rpad, m.d_rowptr.p, m.d_colidx.p, c.d_S32.p, c.d_r32.p,
                           c.d_q32.p, part_c);
    };
    go();
    ERTGB_CUDA(cudaEventRecord(c.ev[0], s));
    for (int r = 0; r < reps; r++) go();
    ERTGB_CUDA(cudaEventRecord(c.ev[1], s));
    ERTGB_CUDA(cudaEventSynchronize(c.ev[1]));
    float t = 0.f;
    ERTGB_CUDA(cudaEventElapsedTime(&t, c.ev[0], c.ev[1]));
    *ms = (double)t / reps;
    *bytes = (double)m.nnz * (4.0 + 4.0 * c.nK) + (double)(n + 1) * 4.0 + 2.0 * n * Rpad * 4.0 + (double)NB * Rpad * 8.0;
    *flops = 2.0 * (double)m.nnz * Rpad + 2.0 * (double)n * Rpad;
}

}  // namespace ertgb
