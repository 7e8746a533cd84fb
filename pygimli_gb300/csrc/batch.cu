// Batched mixed-precision block PCG over independent problems (problems that
// are all FP64 run their own FP64 solves side by side instead).
//
// Every problem of the batch keeps its own context (mesh, matrices of all
// wavenumbers, right-hand sides of all sources, FP64 solution); the batch
// solves all of them with one block PCG whose every kernel covers all
// problems in a single launch.  Each kernel walks a flat list of tiles
// (problem, row block, column chunk) with a persistent grid, so the number
// of launches per iteration does not grow with the number of problems and
// small problems do not leave the GPU idle.  Column scalars (rho, alpha,
// beta, norms) live in flat arrays over all problems' columns; a column's
// block partials sit in its problem's partial block, NB_i row blocks deep.
//
// The recurrence is the mixed-precision one of pcg_mixed.cu with the Jacobi
// preconditioner: FP32 operator and vectors, FP64 reliable updates every
// 64 iterations (x += y, true residual b - A x with the FP64 matrix),
// convergence judged on the FP64 true residual, stalled columns finished by
// the FP64 solver of their own problem.  Iterations are captured 16 at a time
// in a CUDA graph.
//
// The row-block height and the RHS chunk width of the tiles are chosen by an
// autotuner that times the operator kernel on the batch itself for each
// candidate shape and caches the winner per batch signature.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <exception>
#include <map>
#include <thread>
#include <vector>

#include "ertgb_internal.cuh"
#include "reduce.cuh"

namespace ertgb {

namespace {

constexpr int kGraphIters = 16;
constexpr int kReliableEvery = 4;
constexpr int kVecRows = 8;  // rows per pass of a vector tile (block 32 x 8)
// iterations of the FP32 phase; columns still active then finish in FP64
// (FP32 cannot resolve the smallest-wavenumber systems, whose FP32 rounding
// reaches their smallest eigenvalue, and some of them creep rather than stall)
constexpr int kFp32Cap = 6144;

struct BProb {
    int64_t n, nnz, R, Rpad;
    int nE, nK, NB;
    int64_t col0, poff;  // first batch column, first partial element
    const int32_t *rowptr, *colidx;
    const float *S32, *dinv32;
    const double *S, *b, *pnorm2;
    double *x;
    float *r, *p, *q, *y;
};

struct Tile {
    int32_t prob, rb, cb;  // problem, row block, column block (32 * width columns)
};

// --------------------------------------------------------------- vectors
__global__ void kb_init(int ntiles, const Tile *__restrict__ tiles, const BProb *__restrict__ P, int RB,
                        double *__restrict__ pa, double *__restrict__ pb) {
    __shared__ double sa[kVecRows][32], sb[kVecRows][32];
    for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
        const Tile tl = tiles[it];
        const BProb pr = P[tl.prob];
        const int64_t t = (int64_t)tl.cb * 32 + threadIdx.x;
        const int64_t ki = t < pr.R ? t / pr.nE : 0;
        const float *dk = pr.dinv32 + ki * pr.n;
        const int64_t r0 = (int64_t)tl.rb * RB, r1 = min(pr.n, r0 + RB);
        float a = 0.f;
        double bb = 0.0;
        for (int64_t row = r0 + threadIdx.y; row < r1; row += kVecRows) {
            const int64_t i = row * pr.Rpad + t;
            const double bv = pr.b[i];
            const float rv = (float)bv;
            const float z = t < pr.R ? rv * dk[row] : 0.f;
            pr.r[i] = rv;
            pr.p[i] = z;
            pr.y[i] = 0.f;
            a = fmaf(rv, z, a);
            bb = fma(bv, bv, bb);
        }
        sa[threadIdx.y][threadIdx.x] = a;
        sb[threadIdx.y][threadIdx.x] = bb;
        __syncthreads();
        if (threadIdx.y == 0) {
            double s1 = 0.0, s2 = 0.0;
            for (int w = 0; w < kVecRows; w++) {
                s1 += sa[w][threadIdx.x];
                s2 += sb[w][threadIdx.x];
            }
            pa[pr.poff + (int64_t)tl.rb * pr.Rpad + t] = s1;
            pb[pr.poff + (int64_t)tl.rb * pr.Rpad + t] = s2;
        }
        __syncthreads();
    }
}

// y += alpha p, r -= alpha q; partials of r . (dinv r) and r . r
__global__ void kb_update_xr(int ntiles, const Tile *__restrict__ tiles, const BProb *__restrict__ P, int RB,
                             int64_t T, const double *__restrict__ col, const int32_t *__restrict__ active,
                             double *__restrict__ pa, double *__restrict__ pb) {
    __shared__ double sa[kVecRows][32], sb[kVecRows][32];
    for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
        const Tile tl = tiles[it];
        const BProb pr = P[tl.prob];
        const int64_t t = (int64_t)tl.cb * 32 + threadIdx.x;
        const int64_t g = pr.col0 + t;
        const bool act = active[g] != 0;
        const float alpha = (float)col[ALPHA * T + g];
        const int64_t ki = t < pr.R ? t / pr.nE : 0;
        const float *dk = pr.dinv32 + ki * pr.n;
        const int64_t r0 = (int64_t)tl.rb * RB, r1 = min(pr.n, r0 + RB);
        float a = 0.f, b = 0.f;
        if (act) {
            for (int64_t row = r0 + threadIdx.y; row < r1; row += kVecRows) {
                const int64_t i = row * pr.Rpad + t;
                pr.y[i] = fmaf(alpha, pr.p[i], pr.y[i]);
                const float rv = fmaf(-alpha, pr.q[i], pr.r[i]);
                pr.r[i] = rv;
                a = fmaf(rv, rv * dk[row], a);
                b = fmaf(rv, rv, b);
            }
        }
        sa[threadIdx.y][threadIdx.x] = a;
        sb[threadIdx.y][threadIdx.x] = b;
        __syncthreads();
        if (threadIdx.y == 0) {
            double s1 = 0.0, s2 = 0.0;
            for (int w = 0; w < kVecRows; w++) {
                s1 += sa[w][threadIdx.x];
                s2 += sb[w][threadIdx.x];
            }
            pa[pr.poff + (int64_t)tl.rb * pr.Rpad + t] = s1;
            pb[pr.poff + (int64_t)tl.rb * pr.Rpad + t] = s2;
        }
        __syncthreads();
    }
}

__global__ void kb_update_p(int ntiles, const Tile *__restrict__ tiles, const BProb *__restrict__ P, int RB,
                            int64_t T, const double *__restrict__ col, const int32_t *__restrict__ active) {
    for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
        const Tile tl = tiles[it];
        const BProb pr = P[tl.prob];
        const int64_t t = (int64_t)tl.cb * 32 + threadIdx.x;
        const int64_t g = pr.col0 + t;
        if (!active[g]) continue;
        const float beta = (float)col[BETA * T + g];
        const int64_t ki = t < pr.R ? t / pr.nE : 0;
        const float *dk = pr.dinv32 + ki * pr.n;
        const int64_t r0 = (int64_t)tl.rb * RB, r1 = min(pr.n, r0 + RB);
        for (int64_t row = r0 + threadIdx.y; row < r1; row += kVecRows) {
            const int64_t i = row * pr.Rpad + t;
            pr.p[i] = fmaf(beta, pr.p[i], pr.r[i] * dk[row]);
        }
    }
}

// reliable update, part 1: x += y, y = 0
__global__ void kb_accum(int ntiles, const Tile *__restrict__ tiles, const BProb *__restrict__ P, int RB,
                         const int32_t *__restrict__ active, int32_t *__restrict__ nactive) {
    if (blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0) *nactive = 0;
    for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
        const Tile tl = tiles[it];
        const BProb pr = P[tl.prob];
        const int64_t t = (int64_t)tl.cb * 32 + threadIdx.x;
        if (!active[pr.col0 + t]) continue;
        const int64_t r0 = (int64_t)tl.rb * RB, r1 = min(pr.n, r0 + RB);
        for (int64_t row = r0 + threadIdx.y; row < r1; row += kVecRows) {
            const int64_t i = row * pr.Rpad + t;
            pr.x[i] += (double)pr.y[i];
            pr.y[i] = 0.f;
        }
    }
}

// ---------------------------------------------------------------- operator
// q = A_k p (k = wavenumber of the column) on a tile: warp per row, lanes over
// 32 columns x W; partials of p . q
template <int W>
__global__ void __launch_bounds__(256) kb_spmm(int ntiles, const Tile *__restrict__ tiles,
                                               const BProb *__restrict__ P, int RB, double *__restrict__ part) {
    __shared__ double red[8][32 * W];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
        const Tile tl = tiles[it];
        const BProb pr = P[tl.prob];
        const int64_t t0 = (int64_t)tl.cb * 32 * W + lane;
        int64_t kofs[W];
#pragma unroll
        for (int j = 0; j < W; j++) kofs[j] = min((t0 + 32 * j) / pr.nE, (int64_t)pr.nK - 1) * pr.nnz;
        float dot[W];
#pragma unroll
        for (int j = 0; j < W; j++) dot[j] = 0.f;
        const int64_t r0 = (int64_t)tl.rb * RB, r1 = min(pr.n, r0 + RB);
        for (int64_t row = r0 + wid; row < r1; row += 8) {
            float acc[W];
#pragma unroll
            for (int j = 0; j < W; j++) acc[j] = 0.f;
            const int32_t s1 = pr.rowptr[row + 1];
#pragma unroll 4
            for (int32_t s = pr.rowptr[row]; s < s1; s++) {
                const int64_t c = pr.colidx[s];
                const float *pc = pr.p + c * pr.Rpad + t0;
#pragma unroll
                for (int j = 0; j < W; j++) acc[j] = fmaf(pr.S32[kofs[j] + s], __ldg(pc + 32 * j), acc[j]);
            }
            float *qr = pr.q + row * pr.Rpad + t0;
            const float *prow = pr.p + row * pr.Rpad + t0;
#pragma unroll
            for (int j = 0; j < W; j++) {
                qr[32 * j] = acc[j];
                dot[j] = fmaf(prow[32 * j], acc[j], dot[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < W; j++) red[wid][lane + 32 * j] = (double)dot[j];
        __syncthreads();
        for (int c = threadIdx.x; c < 32 * W; c += blockDim.x) {
            double s = 0.0;
#pragma unroll
            for (int w = 0; w < 8; w++) s += red[w][c];
            part[pr.poff + (int64_t)tl.rb * pr.Rpad + (int64_t)tl.cb * 32 * W + c] = s;
        }
        __syncthreads();
    }
}

// reliable update, part 2: true residual r = b - A x in FP64, r32 restarted
// from it; partials of r32 . (dinv r32) and ||r||^2
template <int W>
__global__ void __launch_bounds__(256) kb_residual(int ntiles, const Tile *__restrict__ tiles,
                                                   const BProb *__restrict__ P, int RB,
                                                   const int32_t *__restrict__ active, double *__restrict__ pa,
                                                   double *__restrict__ pb) {
    __shared__ double ra[8][32 * W], rb[8][32 * W];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int it = blockIdx.x; it < ntiles; it += gridDim.x) {
        const Tile tl = tiles[it];
        const BProb pr = P[tl.prob];
        const int64_t t0 = (int64_t)tl.cb * 32 * W + lane;
        int64_t kofs[W], kdi[W];
        bool act[W];
#pragma unroll
        for (int j = 0; j < W; j++) {
            const int64_t t = t0 + 32 * j;
            const int64_t ki = min(t / pr.nE, (int64_t)pr.nK - 1);
            kofs[j] = ki * pr.nnz;
            kdi[j] = ki * pr.n;
            act[j] = active[pr.col0 + t] != 0;
        }
        double sa[W], sb[W];
#pragma unroll
        for (int j = 0; j < W; j++) sa[j] = sb[j] = 0.0;
        const int64_t r0 = (int64_t)tl.rb * RB, r1 = min(pr.n, r0 + RB);
        for (int64_t row = r0 + wid; row < r1; row += 8) {
            double acc[W];
#pragma unroll
            for (int j = 0; j < W; j++) acc[j] = 0.0;
            const int32_t s1 = pr.rowptr[row + 1];
            for (int32_t s = pr.rowptr[row]; s < s1; s++) {
                const int64_t c = pr.colidx[s];
                const double *xc = pr.x + c * pr.Rpad + t0;
#pragma unroll
                for (int j = 0; j < W; j++)
                    if (act[j]) acc[j] = fma(pr.S[kofs[j] + s], xc[32 * j], acc[j]);
            }
#pragma unroll
            for (int j = 0; j < W; j++) {
                if (!act[j]) continue;
                const int64_t i = row * pr.Rpad + t0 + 32 * j;
                const double rv = pr.b[i] - acc[j];
                const float r = (float)rv;
                pr.r[i] = r;
                sa[j] += (double)(r * (r * pr.dinv32[kdi[j] + row]));
                sb[j] = fma(rv, rv, sb[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < W; j++) {
            ra[wid][lane + 32 * j] = sa[j];
            rb[wid][lane + 32 * j] = sb[j];
        }
        __syncthreads();
        for (int c = threadIdx.x; c < 32 * W; c += blockDim.x) {
            double s1 = 0.0, s2 = 0.0;
#pragma unroll
            for (int w = 0; w < 8; w++) {
                s1 += ra[w][c];
                s2 += rb[w][c];
            }
            const int64_t off = pr.poff + (int64_t)tl.rb * pr.Rpad + (int64_t)tl.cb * 32 * W + c;
            pa[off] = s1;
            pb[off] = s2;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------ column scalars
// block (32, 32) per 32 columns of the batch; column g of problem cprob[g]
struct ColView {
    const BProb *P;
    const int32_t *cprob;
    int64_t T;
};

__device__ inline double bcol_sum(const ColView &v, const double *part, int64_t g, double (*red)[33]) {
    const BProb &pr = v.P[v.cprob[g]];
    return col_sum(part + pr.poff, pr.NB, pr.Rpad, g - pr.col0, red);
}

__global__ void kb_finish_init(ColView v, const double *__restrict__ pa, const double *__restrict__ pb,
                               double *__restrict__ col, int32_t *__restrict__ active, int32_t *__restrict__ iters,
                               int32_t *__restrict__ stalled, int32_t *__restrict__ nactive) {
    __shared__ double ra[32][33], rb[32][33];
    const int64_t g = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const double rz = bcol_sum(v, pa, g, ra);
    const double rr = bcol_sum(v, pb, g, rb);
    if (threadIdx.y != 0) return;
    const int64_t T = v.T;
    const BProb &pr = v.P[v.cprob[g]];
    col[RHO * T + g] = rz;
    col[ALPHA * T + g] = 0.0;
    col[BETA * T + g] = 0.0;
    col[BNORM2 * T + g] = pr.pnorm2 ? fmax(rr, kRhsFloor2 * pr.pnorm2[g - pr.col0]) : rr;
    col[RNORM2 * T + g] = rr;
    col[RPREV * T + g] = rr;
    col[STALLS * T + g] = 0.0;
    const int a = (g - pr.col0 < pr.R && rr > 0.0) ? 1 : 0;
    active[g] = a;
    iters[g] = 0;
    stalled[g] = 0;
    if (a) atomicAdd(nactive, 1);
}

// the per-iteration finishes one warp per column (warp_col_sum over the
// column's problem's partial rows)
__global__ void kb_finish_alpha_w(ColView v, const double *__restrict__ part, double *__restrict__ col,
                                  const int32_t *__restrict__ active) {
    const int64_t g = (int64_t)blockIdx.x * kFinWarps + (threadIdx.x >> 5);
    if (g >= v.T) return;
    const BProb &pr = v.P[v.cprob[g]];
    const double pq = warp_col_sum(part + pr.poff, pr.NB, pr.Rpad, g - pr.col0);
    if ((threadIdx.x & 31) != 0 || !active[g]) return;
    col[PQ * v.T + g] = pq;
    col[ALPHA * v.T + g] = (pq != 0.0) ? col[RHO * v.T + g] / pq : 0.0;
}

__global__ void kb_finish_beta_w(ColView v, const double *__restrict__ pa, double *__restrict__ col,
                                 const int32_t *__restrict__ active, int32_t *__restrict__ iters) {
    const int64_t g = (int64_t)blockIdx.x * kFinWarps + (threadIdx.x >> 5);
    if (g >= v.T) return;
    const BProb &pr = v.P[v.cprob[g]];
    const double rz = warp_col_sum(pa + pr.poff, pr.NB, pr.Rpad, g - pr.col0);
    if ((threadIdx.x & 31) != 0) return;
    if (!active[g]) {
        col[BETA * v.T + g] = 0.0;
        return;
    }
    iters[g] += 1;
    const double rho = col[RHO * v.T + g];
    col[BETA * v.T + g] = (rho != 0.0 && rz == rz) ? rz / rho : 0.0;
    col[RHO * v.T + g] = rz;
}

// reliable update, part 3: FP64 convergence test, rho of the restarted
// residual, stall / divergence detection (the rules of the single-problem
// mixed solver)
__global__ void kb_finish_ru(ColView v, double rtol2, const double *__restrict__ pa, const double *__restrict__ pb,
                             double *__restrict__ col, int32_t *__restrict__ active, int32_t *__restrict__ stalled,
                             int32_t *__restrict__ nactive, int32_t *__restrict__ nstalled) {
    __shared__ double ra[32][33], rb[32][33];
    const int64_t g = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const double rz = bcol_sum(v, pa, g, ra);
    const double rr = bcol_sum(v, pb, g, rb);
    if (threadIdx.y != 0 || !active[g]) return;
    const int64_t T = v.T;
    const double bb = col[BNORM2 * T + g];
    col[RNORM2 * T + g] = rr;
    col[RHO * T + g] = rz;
    if (rr <= rtol2 * bb) {
        active[g] = 0;
        return;
    }
    if (!(rr <= 4.0 * bb) || !(rz == rz)) {
        active[g] = 0;
        stalled[g] = 2;
        atomicAdd(nstalled, 1);
        return;
    }
    const double best = col[RPREV * T + g];
    double stalls = col[STALLS * T + g];
    if (rr < 0.81 * best) {
        col[RPREV * T + g] = rr;
        stalls = 0.0;
    } else {
        stalls += 1.0;
    }
    col[STALLS * T + g] = stalls;
    if (stalls >= 4.0) {
        active[g] = 0;
        stalled[g] = 1;
        atomicAdd(nstalled, 1);
        return;
    }
    atomicAdd(nactive, 1);
}

// end of the FP32 phase: every column still active is handed to FP64
__global__ void kb_cap(int64_t T, int32_t *__restrict__ active, int32_t *__restrict__ stalled,
                       int32_t *__restrict__ nstalled) {
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < T; g += (int64_t)gridDim.x * blockDim.x) {
        if (!active[g]) continue;
        active[g] = 0;
        stalled[g] = 1;
        atomicAdd(nstalled, 1);
    }
}

__global__ void kb_to_f32(int64_t n, const double *__restrict__ a, float *__restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// ---------------------------------------------------------------- host side
struct Shape {
    int RB = 64, W = 1;
};

struct Plan {
    Shape shape;
    std::vector<BProb> probs;
    std::vector<Tile> vtiles, stiles;
    DBuf<BProb> d_probs;
    DBuf<Tile> d_vtiles, d_stiles;
    int64_t T = 0, npart = 0;
};

void build_plan(std::vector<Context *> &cs, const Shape &sh, Plan &pl, cudaStream_t s) {
    pl.shape = sh;
    pl.probs.clear();
    pl.vtiles.clear();
    pl.stiles.clear();
    int64_t col0 = 0, poff = 0;
    for (size_t i = 0; i < cs.size(); i++) {
        Context &c = *cs[i];
        MeshData &m = c.mesh;
        BProb b{};
        b.n = m.n;
        b.nnz = m.nnz;
        b.R = c.R;
        b.Rpad = c.Rpad;
        b.nE = c.nE;
        b.nK = c.nK;
        b.NB = (int)ceil_div(m.n, sh.RB);
        b.col0 = col0;
        b.poff = poff;
        b.rowptr = m.d_rowptr.p;
        b.colidx = m.d_colidx.p;
        b.S32 = c.d_S32.p;
        b.dinv32 = c.d_dinv32.p;
        b.S = c.d_S.p;
        b.b = c.d_r.p;
        b.pnorm2 = c.d_pnorm2.n >= (size_t)c.Rpad ? c.d_pnorm2.p : nullptr;
        b.x = c.d_x.p;
        b.r = c.d_r32.p;
        b.p = c.d_p32.p;
        b.q = c.d_q32.p;
        b.y = c.d_y32.p;
        pl.probs.push_back(b);
        for (int rb = 0; rb < b.NB; rb++) {
            for (int cb = 0; cb < (int)(b.Rpad / 32); cb++) pl.vtiles.push_back(Tile{(int32_t)i, rb, cb});
            for (int cb = 0; cb < (int)(b.Rpad / (32 * sh.W)); cb++) pl.stiles.push_back(Tile{(int32_t)i, rb, cb});
        }
        col0 += b.Rpad;
        poff += (int64_t)b.NB * b.Rpad;
    }
    pl.T = col0;
    pl.npart = poff;
    pl.d_probs.upload(pl.probs, s);
    pl.d_vtiles.upload(pl.vtiles, s);
    pl.d_stiles.upload(pl.stiles, s);
}

int grid_for(int ntiles, int per_sm, int device) {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    return std::max(1, std::min(ntiles, per_sm * std::max(sms, 1)));
}

void launch_spmm(const Plan &pl, int W, int grid, cudaStream_t s, double *part) {
    const int nt = (int)pl.stiles.size();
    switch (W) {
        case 4: kb_spmm<4><<<grid, 256, 0, s>>>(nt, pl.d_stiles.p, pl.d_probs.p, pl.shape.RB, part); break;
        case 2: kb_spmm<2><<<grid, 256, 0, s>>>(nt, pl.d_stiles.p, pl.d_probs.p, pl.shape.RB, part); break;
        default: kb_spmm<1><<<grid, 256, 0, s>>>(nt, pl.d_stiles.p, pl.d_probs.p, pl.shape.RB, part); break;
    }
}

void launch_residual(const Plan &pl, int grid, cudaStream_t s, const int32_t *active, double *pa, double *pb) {
    const int nt = (int)pl.stiles.size();
    switch (pl.shape.W) {
        case 4: kb_residual<4><<<grid, 256, 0, s>>>(nt, pl.d_stiles.p, pl.d_probs.p, pl.shape.RB, active, pa, pb); break;
        case 2: kb_residual<2><<<grid, 256, 0, s>>>(nt, pl.d_stiles.p, pl.d_probs.p, pl.shape.RB, active, pa, pb); break;
        default: kb_residual<1><<<grid, 256, 0, s>>>(nt, pl.d_stiles.p, pl.d_probs.p, pl.shape.RB, active, pa, pb); break;
    }
}

// batch signature -> tuned shape
std::map<std::vector<int64_t>, Shape> g_tuned;

}  // namespace

// Autotuned tile shape of a batch: every (row block, RHS chunk width)
// candidate is timed on the operator kernel of the batch itself.
static Shape tune(std::vector<Context *> &cs, cudaStream_t s, DBuf<double> &part, ertgb_batch_info *out) {
    std::vector<int64_t> key;
    for (Context *c : cs) {
        key.push_back(c->mesh.n);
        key.push_back(c->mesh.nnz);
        key.push_back(c->Rpad);
        key.push_back(c->nK);
    }
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
        if (out) out->cached = 1;
        return it->second;
    }
    Shape best;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    ERTGB_CUDA(cudaEventCreate(&e0));
    ERTGB_CUDA(cudaEventCreate(&e1));
    int cand = 0;
    for (int RB : {32, 64, 128, 256}) {
        for (int W : {1, 2, 4}) {
            bool ok = true;
            for (Context *c : cs) ok = ok && (c->Rpad % (32 * W) == 0);
            if (!ok) continue;
            Plan pl;
            build_plan(cs, Shape{RB, W}, pl, s);
            if (part.n < (size_t)pl.npart) part.alloc((size_t)pl.npart);
            const int grid = grid_for((int)pl.stiles.size(), 8, cs[0]->device);
            launch_spmm(pl, W, grid, s, part.p);  // warm-up
            ERTGB_CUDA(cudaEventRecord(e0, s));
            for (int r = 0; r < 3; r++) launch_spmm(pl, W, grid, s, part.p);
            ERTGB_CUDA(cudaEventRecord(e1, s));
            ERTGB_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            ERTGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            ms /= 3.f;
            if (out && cand < 16) {
                out->cand_rows[cand] = RB;
                out->cand_width[cand] = 32 * W;
                out->cand_ms[cand] = ms;
            }
            cand++;
            if (ms < best_ms) {
                best_ms = ms;
                best = Shape{RB, W};
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (out) {
        out->n_candidates = std::min(cand, 16);
        out->cached = 0;
    }
    g_tuned[key] = best;
    return best;
}

namespace {

// Every problem in FP64 (the problems' own precision): the FP64 block PCG of
// each problem with its own preconditioner, all problems side by side, each
// on its own stream and host thread (there is no FP32 phase to share).
int batch_solve_fp64(std::vector<Context *> &cs, cudaStream_t s, ertgb_batch_info *tuning) {
    cudaEvent_t ready;
    ERTGB_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
    ERTGB_CUDA(cudaEventRecord(ready, s));
    std::vector<int> rcs(cs.size(), ERTGB_OK);
    std::vector<std::exception_ptr> errs(cs.size());
    std::vector<std::thread> th;
    for (size_t f = 0; f < cs.size(); f++) {
        th.emplace_back([&, f] {
            try {
                Context &c = *cs[f];
                ERTGB_CUDA(cudaSetDevice(c.device));
                ERTGB_CUDA(cudaStreamWaitEvent(c.stream, ready, 0));
                rcs[f] = pcg_solve(c, c.stream);
                ERTGB_CUDA(cudaStreamSynchronize(c.stream));
            } catch (...) {
                errs[f] = std::current_exception();
            }
        });
    }
    for (auto &t : th) t.join();
    cudaEventDestroy(ready);
    for (auto &e : errs)
        if (e) std::rethrow_exception(e);
    int status = ERTGB_OK, maxit = 0;
    int64_t cols = 0;
    for (size_t f = 0; f < cs.size(); f++) {
        if (rcs[f] != ERTGB_OK) status = rcs[f];
        maxit = std::max(maxit, cs[f]->stats.iterations);
        cols += cs[f]->Rpad;
    }
    if (tuning) {
        tuning->iterations = maxit;
        tuning->columns = cols;
    }
    return status;
}

}  // namespace

int batch_solve(std::vector<Context *> &cs, cudaStream_t s, ertgb_batch_info *tuning, int *stalled_out) {
    bool all_fp64 = true;
    for (Context *c : cs) all_fp64 = all_fp64 && c->precision == ERTGB_PRECISION_FP64;
    if (all_fp64) {
        if (stalled_out) *stalled_out = 0;
        return batch_solve_fp64(cs, s, tuning);
    }
    // per-problem FP32 operands and recurrence vectors
    for (Context *cp : cs) {
        Context &c = *cp;
        MeshData &m = c.mesh;
        c.d_x.alloc((size_t)m.n * c.Rpad);
        c.d_S32.alloc((size_t)c.nK * m.nnz);
        c.d_dinv32.alloc((size_t)c.nK * m.n);
        c.d_r32.alloc((size_t)m.n * c.Rpad);
        c.d_p32.alloc((size_t)m.n * c.Rpad);
        c.d_q32.alloc((size_t)m.n * c.Rpad);
        c.d_y32.alloc((size_t)m.n * c.Rpad);
        ERTGB_CUDA(cudaMemsetAsync(c.d_x.p, 0, sizeof(double) * m.n * c.Rpad, s));
        ERTGB_CUDA(cudaMemsetAsync(c.d_p32.p, 0, sizeof(float) * m.n * c.Rpad, s));
        kb_to_f32<<<(unsigned)std::min<int64_t>(ceil_div((int64_t)c.nK * m.nnz, 256), 4096), 256, 0, s>>>(
            (int64_t)c.nK * m.nnz, c.d_S.p, c.d_S32.p);
        kb_to_f32<<<(unsigned)std::min<int64_t>(ceil_div((int64_t)c.nK * m.n, 256), 4096), 256, 0, s>>>(
            (int64_t)c.nK * m.n, c.d_dinv.p, c.d_dinv32.p);
        ERTGB_CUDA(cudaGetLastError());
    }
    DBuf<double> part_a, part_b, part_c;
    const Shape sh = tune(cs, s, part_c, tuning);
    Plan pl;
    build_plan(cs, sh, pl, s);
    if (tuning) {
        tuning->rows_per_tile = sh.RB;
        tuning->rhs_width = 32 * sh.W;
        tuning->spmm_tiles = (int64_t)pl.stiles.size();
        tuning->vector_tiles = (int64_t)pl.vtiles.size();
        tuning->columns = pl.T;
    }
    part_a.alloc((size_t)pl.npart);
    part_b.alloc((size_t)pl.npart);
    if (part_c.n < (size_t)pl.npart) part_c.alloc((size_t)pl.npart);
    const int64_t T = pl.T;
    DBuf<double> col;
    col.alloc((size_t)NCOL * T);
    DBuf<int32_t> state;
    state.alloc((size_t)3 * T + 2);
    int32_t *active = state.p, *iters = state.p + T, *stalled = state.p + 2 * T, *nactive = state.p + 3 * T,
            *nstalled = state.p + 3 * T + 1;
    ERTGB_CUDA(cudaMemsetAsync(nactive, 0, 2 * sizeof(int32_t), s));
    DBuf<int32_t> cprob;
    {
        std::vector<int32_t> cp((size_t)T);
        for (size_t i = 0; i < pl.probs.size(); i++)
            for (int64_t t = 0; t < pl.probs[i].Rpad; t++) cp[(size_t)(pl.probs[i].col0 + t)] = (int32_t)i;
        cprob.upload(cp, s);
    }
    const ColView cv{pl.d_probs.p, cprob.p, T};
    const int nv = (int)pl.vtiles.size();
    const int gv = grid_for(nv, 16, cs[0]->device), gs = grid_for((int)pl.stiles.size(), 8, cs[0]->device);
    const dim3 vb(32, kVecRows), fb(32, 32), fg((unsigned)(T / 32));
    const unsigned fwg = (unsigned)ceil_div(T, kFinWarps);
    const Tile *vt = pl.d_vtiles.p;
    const BProb *pp = pl.d_probs.p;
    const int RB = sh.RB;
    double rtol = 0.0;
    int max_iter = 1 << 30;
    for (Context *c : cs) {
        rtol = std::max(rtol, c->rtol);
        max_iter = std::min(max_iter, c->max_iter);
    }
    const double rtol2 = rtol * rtol;
    kb_init<<<gv, vb, 0, s>>>(nv, vt, pp, RB, part_a.p, part_b.p);
    kb_finish_init<<<fg, fb, 0, s>>>(cv, part_a.p, part_b.p, col.p, active, iters, stalled, nactive);
    ERTGB_CUDA(cudaGetLastError());

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
            launch_spmm(pl, sh.W, gs, s, part_c.p);
            kb_finish_alpha_w<<<fwg, 32 * kFinWarps, 0, s>>>(cv, part_c.p, col.p, active);
            kb_update_xr<<<gv, vb, 0, s>>>(nv, vt, pp, RB, T, col.p, active, part_a.p, part_b.p);
            kb_finish_beta_w<<<fwg, 32 * kFinWarps, 0, s>>>(cv, part_a.p, col.p, active, iters);
            kb_update_p<<<gv, vb, 0, s>>>(nv, vt, pp, RB, T, col.p, active);
        }
        ERTGB_CUDA(cudaStreamEndCapture(s, &g_it));
        ERTGB_CUDA(cudaGraphInstantiate(&e_it, g_it, 0));
        ERTGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        kb_accum<<<gv, vb, 0, s>>>(nv, vt, pp, RB, active, nactive);
        launch_residual(pl, gs, s, active, part_a.p, part_b.p);
        kb_finish_ru<<<fg, fb, 0, s>>>(cv, rtol2, part_a.p, part_b.p, col.p, active, stalled, nactive, nstalled);
        ERTGB_CUDA(cudaStreamEndCapture(s, &g_ru));
        ERTGB_CUDA(cudaGraphInstantiate(&e_ru, g_ru, 0));
        int32_t h_active = 0;
        ERTGB_CUDA(cudaMemcpyAsync(&h_active, nactive, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        ERTGB_CUDA(cudaStreamSynchronize(s));
        while (h_active > 0) {
            if (iterations >= std::min(max_iter, kFp32Cap)) {
                if (iterations >= max_iter) {
                    status = ERTGB_NOT_CONVERGED;
                } else {
                    kb_cap<<<(unsigned)ceil_div(T, 256), 256, 0, s>>>(T, active, stalled, nstalled);
                    ERTGB_CUDA(cudaGetLastError());
                }
                break;
            }
            for (int u = 0; u < kReliableEvery; u++) ERTGB_CUDA(cudaGraphLaunch(e_it, s));
            iterations += kReliableEvery * kGraphIters;
            ERTGB_CUDA(cudaGraphLaunch(e_ru, s));
            ERTGB_CUDA(cudaMemcpyAsync(&h_active, nactive, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            ERTGB_CUDA(cudaStreamSynchronize(s));
        }
    } catch (...) {
        cudaStreamEndCapture(s, &g_it);
        cleanup();
        throw;
    }
    cleanup();
    if (tuning) {
        tuning->iterations = iterations;
        tuning->launches = (int64_t)(iterations / (kReliableEvery * kGraphIters)) *
                               (5 * kGraphIters * kReliableEvery + 3) + 2;
    }
    // per problem: statistics, FP64 finish of stalled columns
    std::vector<int32_t> it_h((size_t)T), st_h((size_t)T);
    std::vector<double> rn((size_t)T), bn((size_t)T);
    ERTGB_CUDA(cudaMemcpyAsync(it_h.data(), iters, sizeof(int32_t) * T, cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaMemcpyAsync(st_h.data(), stalled, sizeof(int32_t) * T, cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaMemcpyAsync(rn.data(), col.p + RNORM2 * T, sizeof(double) * T, cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaMemcpyAsync(bn.data(), col.p + BNORM2 * T, sizeof(double) * T, cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    int total_stalled = 0;
    std::vector<size_t> fallback;
    for (size_t i = 0; i < cs.size(); i++) {
        Context &c = *cs[i];
        const BProb &b = pl.probs[i];
        int maxit = 0, nst = 0;
        double maxres = 0.0;
        for (int64_t t = 0; t < b.R; t++) {
            const size_t g = (size_t)(b.col0 + t);
            maxit = std::max(maxit, it_h[g]);
            nst += st_h[g] != 0;
            if (bn[g] > 0) maxres = std::max(maxres, std::sqrt(rn[g] / bn[g]));
        }
        c.stats.iterations = maxit;
        c.stats.n_rhs = (int32_t)c.R;
        c.stats.max_rel_residual = maxres;
        c.stats.stalled_columns = nst;
        if (status == ERTGB_OK && nst > 0) {
            // the FP64 solver warm-starts from the context's own column state
            // (scalars with the right-hand-side norms, flags, iteration
            // counts, stalled mask): hand it this problem's slice of the batch
            total_stalled += nst;
            const int64_t Rp = b.Rpad;
            c.d_col.alloc((size_t)NCOL * Rp);
            c.d_active.alloc(ColState::size(Rp));
            for (int slot = 0; slot < NCOL; slot++)
                ERTGB_CUDA(cudaMemcpyAsync(c.d_col.p + (size_t)slot * Rp, col.p + (size_t)slot * T + b.col0,
                                           sizeof(double) * Rp, cudaMemcpyDeviceToDevice, s));
            ColState own(c.d_active.p, Rp);
            ERTGB_CUDA(cudaMemcpyAsync(own.active, active + b.col0, sizeof(int32_t) * Rp, cudaMemcpyDeviceToDevice, s));
            ERTGB_CUDA(cudaMemcpyAsync(own.iters, iters + b.col0, sizeof(int32_t) * Rp, cudaMemcpyDeviceToDevice, s));
            ERTGB_CUDA(cudaMemcpyAsync(own.stalled, stalled + b.col0, sizeof(int32_t) * Rp, cudaMemcpyDeviceToDevice, s));
            ERTGB_CUDA(cudaMemsetAsync(own.nactive, 0, 2 * sizeof(int32_t), s));
            pcg_prepare(c);
            fallback.push_back(i);
        }
    }
    if (!fallback.empty()) {
        // FP64 finish of the stalled columns: every problem on its own stream
        // and host thread, so the problems' solves run side by side
        cudaEvent_t ready;
        ERTGB_CUDA(cudaEventCreateWithFlags(&ready, cudaEventDisableTiming));
        ERTGB_CUDA(cudaEventRecord(ready, s));
        std::vector<int> rcs(fallback.size(), ERTGB_OK);
        std::vector<std::exception_ptr> errs(fallback.size());
        std::vector<std::thread> th;
        for (size_t f = 0; f < fallback.size(); f++) {
            th.emplace_back([&, f] {
                try {
                    Context &c = *cs[fallback[f]];
                    ERTGB_CUDA(cudaSetDevice(c.device));
                    ERTGB_CUDA(cudaStreamWaitEvent(c.stream, ready, 0));
                    ColState own(c.d_active.p, c.Rpad);
                    rcs[f] = pcg_solve(c, c.stream, own.stalled);
                    ERTGB_CUDA(cudaStreamSynchronize(c.stream));
                } catch (...) {
                    errs[f] = std::current_exception();
                }
            });
        }
        for (auto &t : th) t.join();
        cudaEventDestroy(ready);
        for (auto &e : errs)
            if (e) std::rethrow_exception(e);
        for (int rc : rcs)
            if (rc != ERTGB_OK) status = rc;
    }
    if (stalled_out) *stalled_out = total_stalled;
    return status;
}

}  // namespace ertgb
