// Multi-right-hand-side preconditioned conjugate gradients (FP64).
//
// Replaces the reference's direct solve (CHOLMOD factor per wavenumber, one
// triangular solve per current source: core/src/bert/dcfemmodelling.cpp:
// 2199-2210 and 2285; core/src/cholmodWrapper.cpp:309-420).  All sources of
// all wavenumbers are solved together: the iterate blocks are n x Rpad,
// node-major, column t = k*nE + e uses the matrix of wavenumber k.  Every
// column runs its own CG recurrence (own alpha, beta) and stops when
// ||r_t|| <= rtol ||b_t||; reductions are deterministic (fixed-order block
// partials, no atomics on values).
//
// One iteration = 5 kernels:
//   spmm_dot      q = A p (warp per row, lanes over columns) + partial p.q
//   finish_alpha  alpha_t = rho_t / (p.q)_t
//   update_xr     x += alpha p, r -= alpha q, partial r.z and r.r (z = D^-1 r)
//   finish_beta   convergence test, beta_t = (r.z)_t / rho_t
//   update_p      p = D^-1 r + beta p
// A chunk of iterations is captured once into a CUDA graph and replayed; the
// host reads the count of active columns after each replay.  The iteration
// cap bounds the loop, so the solve never waits on the device indefinitely.
#include <algorithm>
#include <cmath>

#include "ertgb_internal.cuh"
#include "reduce.cuh"

namespace ertgb {

namespace {

constexpr int kRowsPerBlock = 8;  // warps per block in spmm, rows per block in vector kernels
constexpr int kGraphIters = 16;
constexpr int kPartRows = 608;  // block partial rows of every column reduction (4 x 152 SMs)


template <int CH>
__global__ void __launch_bounds__(256) k_spmm_dot(int64_t n, int64_t nnz, int nE, int nK, int64_t Rpad,
                                                  const int32_t *__restrict__ rowptr,
                                                  const int32_t *__restrict__ colidx,
                                                  const double *__restrict__ vals,
                                                  const double *__restrict__ p, double *__restrict__ q,
                                                  double *__restrict__ part, const int32_t *__restrict__ active) {
    __shared__ double red[kRowsPerBlock][32 * CH];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t t0 = (int64_t)blockIdx.y * 32 * CH + lane;
    if (active) {  // a chunk of columns none of which is active has nothing to do (q, partials unused)
        int any = 0;
        for (int c = threadIdx.x; c < 32 * CH; c += blockDim.x) any |= active[(int64_t)blockIdx.y * 32 * CH + c];
        if (!__syncthreads_or(any)) return;
    }
    int64_t kofs[CH];  // value-array offset of each column's wavenumber (padding -> last)
#pragma unroll
    for (int j = 0; j < CH; j++) kofs[j] = min((t0 + 32 * j) / nE, (int64_t)nK - 1) * nnz;
    double dot[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) dot[j] = 0.0;
    for (int64_t row = (int64_t)blockIdx.x * kRowsPerBlock + wid; row < n;
         row += (int64_t)gridDim.x * kRowsPerBlock) {
        double acc[CH];
#pragma unroll
        for (int j = 0; j < CH; j++) acc[j] = 0.0;
        const int32_t s1 = rowptr[row + 1];
        for (int32_t s = rowptr[row]; s < s1; s++) {
            const int64_t col = colidx[s];
            const double *pc = p + col * Rpad + t0;
#pragma unroll
            for (int j = 0; j < CH; j++) acc[j] = fma(vals[kofs[j] + s], pc[32 * j], acc[j]);
        }
        double *qr = q + row * Rpad + t0;
        const double *pr = p + row * Rpad + t0;
#pragma unroll
        for (int j = 0; j < CH; j++) {
            qr[32 * j] = acc[j];
            dot[j] = fma(pr[32 * j], acc[j], dot[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < CH; j++) red[wid][lane + 32 * j] = dot[j];
    __syncthreads();
    for (int c = threadIdx.x; c < 32 * CH; c += blockDim.x) {
        double s = 0.0;
#pragma unroll
        for (int w = 0; w < kRowsPerBlock; w++) s += red[w][c];
        part[(int64_t)blockIdx.x * Rpad + (int64_t)blockIdx.y * 32 * CH + c] = s;
    }
}

// Vector kernels: block (32, 8), grid (Rpad/32, NB); thread column t, rows
// strided by 8*NB.  part_a / part_b receive per-block column partials.
// z (may be null): the preconditioned residual given (IC(0)); null: z = D^-1 r
__global__ void k_init(int64_t n, int nE, int nK, int64_t R, int64_t Rpad, const double *__restrict__ dinv,
                       const double *__restrict__ r, double *__restrict__ p, double *__restrict__ part_a,
                       double *__restrict__ part_b, const double *__restrict__ zg) {
    __shared__ double sa[kRowsPerBlock][32], sb[kRowsPerBlock][32];
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const int64_t ki = t < R ? t / nE : 0;
    const double *dk = dinv + ki * n;
    double a = 0.0, b = 0.0;
    for (int64_t row = (int64_t)blockIdx.y * kRowsPerBlock + threadIdx.y; row < n;
         row += (int64_t)gridDim.y * kRowsPerBlock) {
        const int64_t i = row * Rpad + t;
        const double rv = r[i];
        const double z = t < R ? (zg ? zg[i] : rv * dk[row]) : 0.0;
        p[i] = z;
        a = fma(rv, z, a);
        b = fma(rv, rv, b);
    }
    sa[threadIdx.y][threadIdx.x] = a;
    sb[threadIdx.y][threadIdx.x] = b;
    __syncthreads();
    if (threadIdx.y == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < kRowsPerBlock; w++) {
            s1 += sa[w][threadIdx.x];
            s2 += sb[w][threadIdx.x];
        }
        part_a[(int64_t)blockIdx.y * Rpad + t] = s1;
        part_b[(int64_t)blockIdx.y * Rpad + t] = s2;
    }
}

// BNORM2, the convergence reference, is ||b||^2 raised to kRhsFloor2
// ||S1 u_p / rho_s||^2 (pnorm2, may be null): where the singularity-removal
// right-hand side cancels to rounding noise the solve stops at 1e-3 rtol of
// the primary-field scale instead of chasing the noise.
__global__ void k_finish_init(int64_t Rpad, int64_t R, int NB, const double *__restrict__ part_a,
                              const double *__restrict__ part_b, double *__restrict__ col,
                              int32_t *__restrict__ active, int32_t *__restrict__ iters,
                              int32_t *__restrict__ nactive, const int32_t *__restrict__ mask,
                              const double *__restrict__ pnorm2) {
    __shared__ double ra[32][33], rb[32][33];
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const double rz = col_sum(part_a, NB, Rpad, t, ra);
    const double rr = col_sum(part_b, NB, Rpad, t, rb);
    if (threadIdx.y != 0) return;
    col[RHO * Rpad + t] = rz;
    col[ALPHA * Rpad + t] = 0.0;
    col[BETA * Rpad + t] = 0.0;
    if (mask) {  // warm start of selected columns: keep the right-hand side norms
        if (!mask[t]) return;
        col[RNORM2 * Rpad + t] = rr;
        col[RPREV * Rpad + t] = rr;
        const int a = (rr > 0.0) ? 1 : 0;
        active[t] = a;
        if (a) atomicAdd(nactive, 1);
        return;
    }
    col[BNORM2 * Rpad + t] = pnorm2 ? fmax(rr, kRhsFloor2 * pnorm2[t]) : rr;
    col[RNORM2 * Rpad + t] = rr;
    col[RPREV * Rpad + t] = rr;
    col[STALLS * Rpad + t] = 0.0;
    const int a = (t < R && rr > 0.0) ? 1 : 0;
    active[t] = a;
    iters[t] = 0;
    if (a) atomicAdd(nactive, 1);
}

// Columns marked 2 (diverged in the mixed solver) restart from x = 0.
__global__ void k_zero_restart(int64_t n, int64_t Rpad, const int32_t *__restrict__ mask, double *__restrict__ x) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (mask[t] != 2) return;
    for (int64_t row = (int64_t)blockIdx.y * kRowsPerBlock + threadIdx.y; row < n;
         row += (int64_t)gridDim.y * kRowsPerBlock)
        x[row * Rpad + t] = 0.0;
}

// FP64 residual in place for a warm start: r = b - A x on masked columns
// (warp per row, lanes over columns; each element is read and written by
// the same thread).
template <int CH>
__global__ void __launch_bounds__(256) k_residual64(int64_t n, int64_t nnz, int nE, int nK, int64_t Rpad,
                                                    const int32_t *__restrict__ rowptr,
                                                    const int32_t *__restrict__ colidx,
                                                    const double *__restrict__ vals, const double *__restrict__ x,
                                                    const int32_t *__restrict__ mask, double *__restrict__ rb) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int64_t t0 = (int64_t)blockIdx.y * 32 * CH + lane;
    int64_t kofs[CH];
    bool on[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) {
        kofs[j] = min((t0 + 32 * j) / nE, (int64_t)nK - 1) * nnz;
        on[j] = mask[t0 + 32 * j] != 0;
    }
    for (int64_t row = (int64_t)blockIdx.x * kRowsPerBlock + wid; row < n; row += (int64_t)gridDim.x * kRowsPerBlock) {
        double acc[CH];
#pragma unroll
        for (int j = 0; j < CH; j++) acc[j] = 0.0;
        const int32_t s1 = rowptr[row + 1];
        for (int32_t s = rowptr[row]; s < s1; s++) {
            const int64_t col = colidx[s];
#pragma unroll
            for (int j = 0; j < CH; j++)
                if (on[j]) acc[j] = fma(vals[kofs[j] + s], x[col * Rpad + t0 + 32 * j], acc[j]);
        }
        // (columns restarted from zero have x = 0 here, see k_zero_restart)
#pragma unroll
        for (int j = 0; j < CH; j++)
            if (on[j]) {
                const int64_t i = row * Rpad + t0 + 32 * j;
                rb[i] = rb[i] - acc[j];
            }
    }
}

// alpha = rho / (p . q) per active column, one warp per column (warp_col_sum)
__global__ void k_finish_alpha_w(int64_t Rpad, int NB, const double *__restrict__ part, double *__restrict__ col,
                                 const int32_t *__restrict__ active, int32_t *__restrict__ nactive) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *nactive = 0;
    const int64_t t = (int64_t)blockIdx.x * kFinWarps + (threadIdx.x >> 5);
    if (t >= Rpad) return;  // whole warps
    const double pq = warp_col_sum(part, NB, Rpad, t);
    if ((threadIdx.x & 31) != 0 || !active[t]) return;
    col[PQ * Rpad + t] = pq;
    col[ALPHA * Rpad + t] = (pq != 0.0) ? col[RHO * Rpad + t] / pq : 0.0;
}

__global__ void k_update_xr(int64_t n, int nE, int64_t R, int64_t Rpad, const double *__restrict__ dinv,
                            const double *__restrict__ col, const int32_t *__restrict__ active,
                            double *__restrict__ x, double *__restrict__ r, const double *__restrict__ p,
                            const double *__restrict__ q, double *__restrict__ part_a,
                            double *__restrict__ part_b) {
    __shared__ double sa[kRowsPerBlock][32], sb[kRowsPerBlock][32];
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const bool act = active[t] != 0;
    const double alpha = col[ALPHA * Rpad + t];
    const int64_t ki = t < R ? t / nE : 0;
    const double *dk = dinv ? dinv + ki * n : nullptr;
    double a = 0.0, b = 0.0;
    if (act) {
        for (int64_t row = (int64_t)blockIdx.y * kRowsPerBlock + threadIdx.y; row < n;
             row += (int64_t)gridDim.y * kRowsPerBlock) {
            const int64_t i = row * Rpad + t;
            x[i] = fma(alpha, p[i], x[i]);
            const double rv = fma(-alpha, q[i], r[i]);
            r[i] = rv;
            if (dinv) a = fma(rv, rv * dk[row], a);
            b = fma(rv, rv, b);
        }
    }
    sa[threadIdx.y][threadIdx.x] = a;
    sb[threadIdx.y][threadIdx.x] = b;
    __syncthreads();
    if (threadIdx.y == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < kRowsPerBlock; w++) {
            s1 += sa[w][threadIdx.x];
            s2 += sb[w][threadIdx.x];
        }
        part_a[(int64_t)blockIdx.y * Rpad + t] = s1;
        part_b[(int64_t)blockIdx.y * Rpad + t] = s2;
    }
}

// beta, ||r||^2 and the convergence test per column, one warp per column
__global__ void k_finish_beta_w(int64_t Rpad, int NB, double rtol2, const double *__restrict__ part_a,
                                const double *__restrict__ part_b, double *__restrict__ col,
                                int32_t *__restrict__ active, int32_t *__restrict__ iters,
                                int32_t *__restrict__ nactive) {
    const int64_t t = (int64_t)blockIdx.x * kFinWarps + (threadIdx.x >> 5);
    if (t >= Rpad) return;
    const double rz = warp_col_sum(part_a, NB, Rpad, t);
    const double rr = warp_col_sum(part_b, NB, Rpad, t);
    if ((threadIdx.x & 31) != 0) return;
    if (!active[t]) {
        col[BETA * Rpad + t] = 0.0;
        return;
    }
    iters[t] += 1;
    col[RNORM2 * Rpad + t] = rr;
    const double rho = col[RHO * Rpad + t];
    col[BETA * Rpad + t] = (rho != 0.0) ? rz / rho : 0.0;
    col[RHO * Rpad + t] = rz;
    if (rr <= rtol2 * col[BNORM2 * Rpad + t] || !(rr == rr)) {
        active[t] = 0;
    } else {
        atomicAdd(nactive, 1);
    }
}

__global__ void k_update_p(int64_t n, int nE, int64_t R, int64_t Rpad, const double *__restrict__ dinv,
                           const double *__restrict__ col, const int32_t *__restrict__ active,
                           const double *__restrict__ r, double *__restrict__ p, const double *__restrict__ zg) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (!active[t]) return;
    const double beta = col[BETA * Rpad + t];
    const int64_t ki = t < R ? t / nE : 0;
    const double *dk = dinv ? dinv + ki * n : nullptr;
    for (int64_t row = (int64_t)blockIdx.y * kRowsPerBlock + threadIdx.y; row < n;
         row += (int64_t)gridDim.y * kRowsPerBlock) {
        const int64_t i = row * Rpad + t;
        p[i] = fma(beta, p[i], zg ? zg[i] : r[i] * dk[row]);
    }
}

// column partials of r . z (IC(0): z from the triangular solves)
__global__ void k_dot_rz(int64_t n, int64_t Rpad, const int32_t *__restrict__ active, const double *__restrict__ r,
                         const double *__restrict__ z, double *__restrict__ part_a) {
    __shared__ double sa[kRowsPerBlock][32];
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    double a = 0.0;
    if (active[t]) {
        for (int64_t row = (int64_t)blockIdx.y * kRowsPerBlock + threadIdx.y; row < n;
             row += (int64_t)gridDim.y * kRowsPerBlock) {
            const int64_t i = row * Rpad + t;
            a = fma(r[i], z[i], a);
        }
    }
    sa[threadIdx.y][threadIdx.x] = a;
    __syncthreads();
    if (threadIdx.y == 0) {
        double s1 = 0.0;
        for (int w = 0; w < kRowsPerBlock; w++) s1 += sa[w][threadIdx.x];
        part_a[(int64_t)blockIdx.y * Rpad + t] = s1;
    }
}

int choose_ch(int64_t Rpad) {
    const int64_t w = Rpad / 32;
    for (int ch : {4, 3, 2}) {
        if (w % ch == 0) return ch;
    }
    return 1;
}

// active: skip column chunks without an active column (nullptr: all)
void launch_spmm(int ch, dim3 grid, cudaStream_t s, int64_t n, int64_t nnz, int nE, int nK, int64_t Rpad,
                 const int32_t *rowptr, const int32_t *colidx, const double *vals, const double *p, double *q,
                 double *part, const int32_t *active = nullptr) {
    switch (ch) {
        case 4: k_spmm_dot<4><<<grid, 256, 0, s>>>(n, nnz, nE, nK, Rpad, rowptr, colidx, vals, p, q, part, active); break;
        case 3: k_spmm_dot<3><<<grid, 256, 0, s>>>(n, nnz, nE, nK, Rpad, rowptr, colidx, vals, p, q, part, active); break;
        case 2: k_spmm_dot<2><<<grid, 256, 0, s>>>(n, nnz, nE, nK, Rpad, rowptr, colidx, vals, p, q, part, active); break;
        default: k_spmm_dot<1><<<grid, 256, 0, s>>>(n, nnz, nE, nK, Rpad, rowptr, colidx, vals, p, q, part, active); break;
    }
}

}  // namespace

void pcg_prepare(Context &c) {
    const int64_t n = c.mesh.n, Rpad = c.Rpad;
    const int NB = (int)std::min<int64_t>(ceil_div(n, kRowsPerBlock), kPartRows);
    c.d_p.alloc((size_t)n * Rpad);
    c.d_q.alloc((size_t)n * Rpad);
    c.d_part.alloc((size_t)NB * Rpad * 3);
}

int pcg_solve(Context &c, cudaStream_t s, const int32_t *mask) {
    if (c.precond == ERTGB_PRECOND_BAND && !mask) return band_solve(c, s);  // direct, no iterations
    MeshData &m = c.mesh;
    const int64_t n = m.n, Rpad = c.Rpad, R = c.R;
    const int NB = (int)std::min<int64_t>(ceil_div(n, kRowsPerBlock), kPartRows);
    const int ch = choose_ch(Rpad);
    const int nchunk = (int)(Rpad / (32 * ch));
    // workspaces
    if (!mask) c.d_x.alloc((size_t)n * Rpad);
    c.d_p.alloc((size_t)n * Rpad);
    c.d_q.alloc((size_t)n * Rpad);
    c.d_part.alloc((size_t)NB * Rpad * 3);
    if (!mask) {
        c.d_col.alloc((size_t)NCOL * Rpad);
        c.d_active.alloc(ColState::size(Rpad));
    }
    double *part_a = c.d_part.p, *part_b = c.d_part.p + (size_t)NB * Rpad, *part_c = c.d_part.p + 2 * (size_t)NB * Rpad;
    ColState cs(c.d_active.p, Rpad);
    int32_t *active = cs.active, *iters = cs.iters, *nactive = cs.nactive;
    const dim3 vb(32, kRowsPerBlock), vg((unsigned)(Rpad / 32), (unsigned)NB);
    const dim3 sg((unsigned)NB, (unsigned)nchunk);
    const unsigned fg = (unsigned)(Rpad / 32);
    const dim3 fb(32, 32);
    const unsigned fwg = (unsigned)ceil_div(Rpad, kFinWarps);
    const double rtol2 = c.rtol * c.rtol;
    if (mask) {
        // warm start from x on the masked columns: r = b - A x in place
        k_zero_restart<<<vg, vb, 0, s>>>(n, Rpad, mask, c.d_x.p);
        c.stats.launches_response += 1;
        switch (ch) {
            case 4: k_residual64<4><<<sg, 256, 0, s>>>(n, m.nnz, c.nE, c.nK, Rpad, m.d_rowptr.p, m.d_colidx.p, c.d_S.p, c.d_x.p, mask, c.d_r.p); break;
            case 3: k_residual64<3><<<sg, 256, 0, s>>>(n, m.nnz, c.nE, c.nK, Rpad, m.d_rowptr.p, m.d_colidx.p, c.d_S.p, c.d_x.p, mask, c.d_r.p); break;
            case 2: k_residual64<2><<<sg, 256, 0, s>>>(n, m.nnz, c.nE, c.nK, Rpad, m.d_rowptr.p, m.d_colidx.p, c.d_S.p, c.d_x.p, mask, c.d_r.p); break;
            default: k_residual64<1><<<sg, 256, 0, s>>>(n, m.nnz, c.nE, c.nK, Rpad, m.d_rowptr.p, m.d_colidx.p, c.d_S.p, c.d_x.p, mask, c.d_r.p); break;
        }
        c.stats.launches_response += 1;
    } else {
        ERTGB_CUDA(cudaMemsetAsync(c.d_x.p, 0, sizeof(double) * n * Rpad, s));
    }
    ERTGB_CUDA(cudaMemsetAsync(nactive, 0, sizeof(int32_t), s));
    // IC(0) (plain FP64 solve only; the FP64 finish of the mixed solver keeps Jacobi)
    const bool ic0 = c.precond == ERTGB_PRECOND_IC0 && !mask;
    const double *dv = ic0 ? nullptr : c.d_dinv.p;
    const double *zg = nullptr;
    if (ic0) {
        ic0_setup(c, s);
        c.d_z.alloc((size_t)n * Rpad);
        ic0_apply(c, c.d_r.p, c.d_z.p, s);
        zg = c.d_z.p;
        c.stats.launches_response += ic0_launches(c);
    }
    k_init<<<vg, vb, 0, s>>>(n, c.nE, c.nK, R, Rpad, c.d_dinv.p, c.d_r.p, c.d_p.p, part_a, part_b, zg);
    k_finish_init<<<fg, fb, 0, s>>>(Rpad, R, NB, part_a, part_b, c.d_col.p, active, iters, nactive, mask,
                                    c.d_pnorm2.n >= (size_t)Rpad ? c.d_pnorm2.p : nullptr);
    ERTGB_CUDA(cudaGetLastError());

    // capture a chunk of iterations
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ERTGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int it = 0; it < kGraphIters; it++) {
        launch_spmm(ch, sg, s, n, m.nnz, c.nE, c.nK, Rpad, m.d_rowptr.p, m.d_colidx.p, c.d_S.p, c.d_p.p, c.d_q.p,
                    part_c, active);
        k_finish_alpha_w<<<fwg, 32 * kFinWarps, 0, s>>>(Rpad, NB, part_c, c.d_col.p, active, nactive);
        k_update_xr<<<vg, vb, 0, s>>>(n, c.nE, R, Rpad, dv, c.d_col.p, active, c.d_x.p, c.d_r.p,
                                      c.d_p.p, c.d_q.p, part_a, part_b);
        if (ic0) {
            ic0_apply(c, c.d_r.p, c.d_z.p, s);
            k_dot_rz<<<vg, vb, 0, s>>>(n, Rpad, active, c.d_r.p, c.d_z.p, part_a);
        }
        k_finish_beta_w<<<fwg, 32 * kFinWarps, 0, s>>>(Rpad, NB, rtol2, part_a, part_b, c.d_col.p, active, iters,
                                                       nactive);
        k_update_p<<<vg, vb, 0, s>>>(n, c.nE, R, Rpad, dv, c.d_col.p, active, c.d_r.p, c.d_p.p, zg);
    }
    cudaError_t cap = cudaStreamEndCapture(s, &graph);
    if (cap != cudaSuccess) ERTGB_CUDA(cap);
    cudaError_t inst = cudaGraphInstantiate(&exec, graph, 0);
    if (inst != cudaSuccess) {
        cudaGraphDestroy(graph);
        ERTGB_CUDA(inst);
    }
    c.stats.launches_response += 2;
    int32_t h_active = 0;
    int iterations = 0;
    int status = ERTGB_OK;
    ERTGB_CUDA(cudaMemcpyAsync(&h_active, nactive, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    try {
        while (h_active > 0) {
            if (iterations >= c.max_iter) {
                status = ERTGB_NOT_CONVERGED;
                break;
            }
            ERTGB_CUDA(cudaGraphLaunch(exec, s));
            iterations += kGraphIters;
            c.stats.launches_response += (5 + (ic0 ? ic0_launches(c) + 1 : 0)) * kGraphIters;
            ERTGB_CUDA(cudaMemcpyAsync(&h_active, nactive, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            ERTGB_CUDA(cudaStreamSynchronize(s));
        }
    } catch (...) {
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        throw;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    // statistics: exact iteration count and final relative residual
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
    // with a mask the per-column counts continue those of the mixed solve
    c.stats.iterations = maxit;
    c.stats.max_rel_residual = maxres;
    c.stats.n_rhs = (int32_t)R;
    return status;
}

namespace {
__global__ void k_col_total(int64_t Rpad, int NB, const double *__restrict__ part, double *__restrict__ out) {
    __shared__ double red[32][33];
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const double s = col_sum(part, NB, Rpad, t, red);
    if (threadIdx.y == 0) out[t] = s;
}
}  // namespace

void pcg_finish_init(dim3 g, dim3 b, cudaStream_t s, int64_t Rpad, int64_t R, int NB, const double *pa, const double *pb,
                     double *col, int32_t *active, int32_t *iters, int32_t *nactive, const double *pnorm2) {
    k_finish_init<<<g, b, 0, s>>>(Rpad, R, NB, pa, pb, col, active, iters, nactive, nullptr, pnorm2);
}

int spmm_partial_rows(int64_t n, int cap) { return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, kRowsPerBlock), cap)); }

void spmm_dot_launch(int64_t n, int64_t nnz, const int32_t *rowptr, const int32_t *colidx, const double *vals, int nK,
                     int n_per_k, int64_t ld, const double *X, double *Y, double *dots, double *partials, int NB,
                     cudaStream_t s) {
    const int ch = choose_ch(ld);
    const dim3 sg((unsigned)NB, (unsigned)(ld / (32 * ch)));
    launch_spmm(ch, sg, s, n, nnz, n_per_k, nK, ld, rowptr, colidx, vals, X, Y, partials);
    ERTGB_CUDA(cudaGetLastError());
    k_col_total<<<(unsigned)(ld / 32), dim3(32, 32), 0, s>>>(ld, NB, partials, dots);
    ERTGB_CUDA(cudaGetLastError());
}

void profile_spmm(Context &c, int reps, double *ms, double *bytes, double *flops) {
    MeshData &m = c.mesh;
    const int64_t n = m.n, Rpad = c.Rpad;
    const int NB = (int)std::min<int64_t>(ceil_div(n, kRowsPerBlock), kPartRows);
    const int ch = choose_ch(Rpad);
    const dim3 sg((unsigned)NB, (unsigned)(Rpad / (32 * ch)));
    if (c.d_q.n < (size_t)n * Rpad || c.d_part.n < (size_t)NB * Rpad * 3 || c.d_S.n < (size_t)c.nK * m.nnz)
        throw Error(ERTGB_STATE, "profile needs a completed response");
    cudaStream_t s = c.stream;
    double *part_c = c.d_part.p + 2 * (size_t)NB * Rpad;
    launch_spmm(ch, sg, s, n, m.nnz, c.nE, c.nK, Rpad, m.d_rowptr.p, m.d_colidx.p, c.d_S.p, c.d_x.p, c.d_q.p, part_c);
    ERTGB_CUDA(cudaEventRecord(c.ev[0], s));
    for (int r = 0; r < reps; r++)
        launch_spmm(ch, sg, s, n, m.nnz, c.nE, c.nK, Rpad, m.d_rowptr.p, m.d_colidx.p, c.d_S.p, c.d_x.p, c.d_q.p,
                    part_c);
    ERTGB_CUDA(cudaEventRecord(c.ev[1], s));
    ERTGB_CUDA(cudaEventSynchronize(c.ev[1]));
    float t = 0.f;
    ERTGB_CUDA(cudaEventElapsedTime(&t, c.ev[0], c.ev[1]));
    *ms = (double)t / reps;
    // matrix (column indices + every wavenumber's values), row pointers,
    // p read once, q written once, block partials written
    *bytes = (double)m.nnz * (4.0 + 8.0 * c.nK) + (double)(n + 1) * 4.0 + 2.0 * n * Rpad * 8.0 +
             (double)NB * Rpad * 8.0;
    *flops = 2.0 * (double)m.nnz * Rpad + 2.0 * (double)n * Rpad;
}

}  // namespace ertgb
