// Deterministic per-column reduction of block partials, shared by the
// solver kernels.
#pragma once

#include <cstdint>

namespace ertgb {

// Column reductions: block (32, 32), grid Rpad/32; thread (tx, ty) sums the
// partial rows ty, ty+32, ... of column t, then the 32 sums are added in a
// fixed order (deterministic).  Every thread of the block must call it.
__device__ inline double col_sum(const double *__restrict__ part, int NB, int64_t Rpad, int64_t t,
                                 double (*red)[33]) {
    double s = 0.0;
    for (int b = threadIdx.y; b < NB; b += 32) s += part[(int64_t)b * Rpad + t];
    red[threadIdx.y][threadIdx.x] = s;
    __syncthreads();
    double tot = 0.0;
    if (threadIdx.y == 0)
        for (int w = 0; w < 32; w++) tot += red[w][threadIdx.x];
    return tot;
}

}  // namespace ertgb
