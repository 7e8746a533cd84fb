// Deterministic per-column reduction of block partials, shared by the
// solver kernels.
#pragma once

#include <cstdint>

namespace ertgb {

// Per-column scalar slots of Context::d_col (NCOL x Rpad doubles), shared by
// the FP64 and the mixed-precision solvers.
enum ColSlot { RHO = 0, ALPHA, BETA, BNORM2, RNORM2, PQ, RPREV, STALLS, NCOL };

// Integer per-column state of Context::d_active: active flags, iteration
// counts, stalled flags (Rpad each), then the active and stalled counters.
struct ColState {
    int32_t *active, *iters, *stalled, *nactive, *nstalled;
    ColState(int32_t *base, int64_t Rpad)
        : active(base), iters(base + Rpad), stalled(base + 2 * Rpad), nactive(base + 3 * Rpad),
          nstalled(base + 3 * Rpad + 1) {}
    static size_t size(int64_t Rpad) { return (size_t)Rpad * 3 + 2; }
};

// Column reductions: block (32, 32), grid Rpad/32; thread (tx, ty) sums the
// partial rows ty, ty+32, ... of column t, then warp w adds the 32 sums of
// the block's column w by a shuffle tree (five dependent FP64 additions
// instead of 32: FP64 latency dominates these small kernels) in a fixed order
// (deterministic).  The total is returned to the threads with ty == 0; every
// thread of the block must call it.  red[w][32] holds column w's total.
__device__ inline double col_sum(const double *__restrict__ part, int NB, int64_t Rpad, int64_t t,
                                 double (*red)[33]) {
    // four independent accumulators keep several loads in flight
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int b = threadIdx.y;
    for (; b + 96 < NB; b += 128) {
        s0 += part[(int64_t)b * Rpad + t];
        s1 += part[(int64_t)(b + 32) * Rpad + t];
        s2 += part[(int64_t)(b + 64) * Rpad + t];
        s3 += part[(int64_t)(b + 96) * Rpad + t];
    }
    for (; b < NB; b += 32) s0 += part[(int64_t)b * Rpad + t];
    red[threadIdx.y][threadIdx.x] = (s0 + s1) + (s2 + s3);
    __syncthreads();
    double v = red[threadIdx.x][threadIdx.y];  // warp ty: the 32 sums of column ty
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) red[threadIdx.y][32] = v;
    __syncthreads();
    return threadIdx.y == 0 ? red[threadIdx.x][32] : 0.0;
}

// Column sums of the NB block partials by one warp per column (eight
// columns per block, so the FP64 additions spread over many SMs instead of
// the Rpad / 32 SMs of col_sum): lanes take rows lane, lane + 32, ... in two
// chains, then a shuffle tree; lane 0's total is returned to every lane.
constexpr int kFinWarps = 8;  // columns (warps) per block of the warp-per-column finishes

__device__ __forceinline__ double warp_col_sum(const double *__restrict__ part, int NB, int64_t Rpad, int64_t t) {
    const int lane = threadIdx.x & 31;
    double s0 = 0.0, s1 = 0.0;
    int b = lane;
    for (; b + 32 < NB; b += 64) {
        s0 += part[(int64_t)b * Rpad + t];
        s1 += part[(int64_t)(b + 32) * Rpad + t];
    }
    if (b < NB) s0 += part[(int64_t)b * Rpad + t];
    double v = s0 + s1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return __shfl_sync(0xffffffffu, v, 0);
}

}  // namespace ertgb
