// Regularised Gauss-Newton model update on the GPU: the CGLS solver of
// pyGIMLi's inversion (solveCGLSCDWWhtrans, core/src/solver.cpp:27-212),
// called by RInversion::oneStep (core/src/inversion.cpp:249-372), solving
//
//   (J_t^T Wd^2 J_t + lambda (Wc C Wm)^T (Wc C Wm)) dx = J_t^T Wd^2 b - lambda (Wc C Wm)^T roughness
//
// with J_t = diag(td) J diag(1/tm) (data / model transformation derivatives),
// in the reference's order of operations, including its rounding of C p to
// 1e-10.  J stays where createJacobian left it (FP64 or FP32, row-major
// D x P); every product with J streams it once from HBM:
//   J x     block per datum row, fixed-order block reduction;
//   J^T y   thread per model column over a segment of rows, segments summed
//           in a fixed order.
// The constraint matrix C (and its transpose) is CSR FP64.  Vectors and
// scalars are FP64; the dot products are deterministic two-stage reductions
// whose results the host reads every iteration (two syncs per iteration,
// small against the two passes over J).  With an FP32 Jacobian the products
// run in FP32 (per-thread partial sums) and are summed in FP64.
#include <algorithm>
#include <cmath>
#include <vector>

#include "ertgb_internal.cuh"

namespace ertgb {

namespace {

constexpr int kThreads = 256;
constexpr int kRowSeg = 16;  // row segments of the J^T products

template <typename T>
__global__ void k_jmul(int64_t D, int64_t P, const T *__restrict__ J, const double *__restrict__ x,
                       const double *__restrict__ scale, double *__restrict__ y) {
    __shared__ double red[kThreads];
    for (int64_t d = blockIdx.x; d < D; d += gridDim.x) {
        const T *row = J + d * P;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
        int64_t p = threadIdx.x;
        for (; p + 3 * kThreads < P; p += 4 * kThreads) {
            a0 = fma((double)row[p], x[p], a0);
            a1 = fma((double)row[p + kThreads], x[p + kThreads], a1);
            a2 = fma((double)row[p + 2 * kThreads], x[p + 2 * kThreads], a2);
            a3 = fma((double)row[p + 3 * kThreads], x[p + 3 * kThreads], a3);
        }
        for (; p < P; p += kThreads) a0 = fma((double)row[p], x[p], a0);
        red[threadIdx.x] = (a0 + a1) + (a2 + a3);
        __syncthreads();
        for (int w = kThreads / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) y[d] = scale ? red[0] * scale[d] : red[0];
        __syncthreads();
    }
}

// part[s][p] = sum over rows of segment s of J[d][p] y[d]
template <typename T>
__global__ void k_jtmul(int64_t D, int64_t P, const T *__restrict__ J, const double *__restrict__ y,
                        double *__restrict__ part) {
    const int64_t p = blockIdx.x * (int64_t)kThreads + threadIdx.x;
    const int64_t seg = (D + gridDim.y - 1) / gridDim.y;
    const int64_t d0 = blockIdx.y * seg, d1 = min(D, d0 + seg);
    if (p >= P) return;
    double a0 = 0.0, a1 = 0.0;
    int64_t d = d0;
    for (; d + 1 < d1; d += 2) {
        a0 = fma((double)J[d * P + p], y[d], a0);
        a1 = fma((double)J[(d + 1) * P + p], y[d + 1], a1);
    }
    if (d < d1) a0 = fma((double)J[d * P + p], y[d], a0);
    part[(int64_t)blockIdx.y * P + p] = a0 + a1;
}

// FP32 Jacobian: products in FP32 (float4 loads of J and of an FP32 copy of
// the vector), per-thread FP32 partial sums, FP64 across threads and
// segments.  GB300's FP64 pipe (1/55 of FP32) would otherwise bound the pass,
// not HBM.
__global__ void k_jmul32(int64_t D, int64_t P, const float *__restrict__ J, const float *__restrict__ x,
                         const double *__restrict__ scale, double *__restrict__ y) {
    __shared__ double red[kThreads];
    const int64_t P4 = P / 4;
    for (int64_t d = blockIdx.x; d < D; d += gridDim.x) {
        const float *row = J + d * P;
        float a0 = 0.f, a1 = 0.f;
        // rows start 16-byte aligned only when P is a multiple of 4
        if ((P & 3) == 0) {
            const float4 *r4 = reinterpret_cast<const float4 *>(row);
            const float4 *x4 = reinterpret_cast<const float4 *>(x);
            int64_t p = threadIdx.x;
            for (; p + kThreads < P4; p += 2 * kThreads) {
                const float4 j0 = __ldg(r4 + p), j1 = __ldg(r4 + p + kThreads);
                const float4 v0 = x4[p], v1 = x4[p + kThreads];
                a0 = fmaf(j0.x, v0.x, fmaf(j0.y, v0.y, fmaf(j0.z, v0.z, fmaf(j0.w, v0.w, a0))));
                a1 = fmaf(j1.x, v1.x, fmaf(j1.y, v1.y, fmaf(j1.z, v1.z, fmaf(j1.w, v1.w, a1))));
            }
            for (; p < P4; p += kThreads) {
                const float4 j0 = __ldg(r4 + p);
                const float4 v0 = x4[p];
                a0 = fmaf(j0.x, v0.x, fmaf(j0.y, v0.y, fmaf(j0.z, v0.z, fmaf(j0.w, v0.w, a0))));
            }
        } else {
            for (int64_t p = threadIdx.x; p < P; p += kThreads) a0 = fmaf(__ldg(row + p), x[p], a0);
        }
        red[threadIdx.x] = (double)a0 + (double)a1;
        __syncthreads();
        for (int w = kThreads / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) y[d] = scale ? red[0] * scale[d] : red[0];
        __syncthreads();
    }
}

// part[s][p] for 4 consecutive columns per thread (P a multiple of 4)
__global__ void k_jtmul32(int64_t D, int64_t P, const float *__restrict__ J, const float *__restrict__ y,
                          double *__restrict__ part) {
    const int64_t q = blockIdx.x * (int64_t)kThreads + threadIdx.x;  // float4 column group
    const int64_t seg = (D + gridDim.y - 1) / gridDim.y;
    const int64_t d0 = blockIdx.y * seg, d1 = min(D, d0 + seg);
    if (q * 4 >= P) return;
    const float4 *J4 = reinterpret_cast<const float4 *>(J);
    const int64_t P4 = P / 4;
    float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = make_float4(0.f, 0.f, 0.f, 0.f);
    int64_t d = d0;
    for (; d + 1 < d1; d += 2) {
        const float4 j0 = __ldg(J4 + d * P4 + q), j1 = __ldg(J4 + (d + 1) * P4 + q);
        const float y0 = y[d], y1 = y[d + 1];
        a.x = fmaf(j0.x, y0, a.x); a.y = fmaf(j0.y, y0, a.y); a.z = fmaf(j0.z, y0, a.z); a.w = fmaf(j0.w, y0, a.w);
        b.x = fmaf(j1.x, y1, b.x); b.y = fmaf(j1.y, y1, b.y); b.z = fmaf(j1.z, y1, b.z); b.w = fmaf(j1.w, y1, b.w);
    }
    if (d < d1) {
        const float4 j0 = __ldg(J4 + d * P4 + q);
        const float y0 = y[d];
        a.x = fmaf(j0.x, y0, a.x); a.y = fmaf(j0.y, y0, a.y); a.z = fmaf(j0.z, y0, a.z); a.w = fmaf(j0.w, y0, a.w);
    }
    double *o = part + (int64_t)blockIdx.y * P + q * 4;
    o[0] = (double)a.x + (double)b.x;
    o[1] = (double)a.y + (double)b.y;
    o[2] = (double)a.z + (double)b.z;
    o[3] = (double)a.w + (double)b.w;
}

__global__ void k_to32(int64_t n, const double *__restrict__ a, float *__restrict__ b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}

// out[p] = (sum_s part[s][p]) / div[p] (div may be null)
__global__ void k_seg_sum(int64_t P, int S, const double *__restrict__ part, const double *__restrict__ div,
                          double *__restrict__ out) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < P; p += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < S; k++) s += part[(int64_t)k * P + p];
        out[p] = div ? s / div[p] : s;
    }
}

// y[r] = sum_j C[r][j] (w[j] x[j]) (w may be null), optionally rounded to 1e-10
__global__ void k_csr_mul(int64_t R, const int32_t *__restrict__ rowptr, const int32_t *__restrict__ cols,
                          const double *__restrict__ vals, const double *__restrict__ x, const double *__restrict__ w,
                          int round10, double *__restrict__ y) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < R; r += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int32_t q = rowptr[r]; q < rowptr[r + 1]; q++) {
            const int32_t j = cols[q];
            s += vals[q] * (w ? w[j] * x[j] : x[j]);
        }
        y[r] = round10 ? rint(s / 1e-10) * 1e-10 : s;
    }
}

// generic elementwise: out = a * (b ? b : 1) * (c ? c : 1) * (d ? d : 1)
__global__ void k_mul4(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                       const double *__restrict__ c, const double *__restrict__ d, double *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double v = a[i];
        if (b) v *= b[i];
        if (c) v *= c[i];
        if (d) v *= d[i];
        out[i] = v;
    }
}

__global__ void k_div(int64_t n, const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = a[i] / b[i];
}

// r = jt - lambda * ctc * wm - cdx
__global__ void k_rvec(int64_t n, const double *__restrict__ jt, const double *__restrict__ ctc,
                       const double *__restrict__ wm, double lambda, const double *__restrict__ cdx,
                       double *__restrict__ r) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r[i] = jt[i] - ctc[i] * wm[i] * lambda - cdx[i];
}

// y += a x
__global__ void k_axpy(int64_t n, double a, const double *__restrict__ x, double *__restrict__ y) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fma(a, x[i], y[i]);
}

// x *= a
__global__ void k_scale(int64_t n, double a, double *__restrict__ x) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= a;
}

// p = r + b p
__global__ void k_xpby(int64_t n, const double *__restrict__ r, double b, double *__restrict__ p) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        p[i] = r[i] + b * p[i];
}

// dot products, stage 1: block partials
__global__ void k_dot(int64_t n, const double *__restrict__ a, const double *__restrict__ b, double *__restrict__ part) {
    __shared__ double red[kThreads];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s = fma(a[i], b[i], s);
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// stage 2: one block sums the partials in a fixed order
__global__ void k_dot_final(int nb, const double *__restrict__ part, double *__restrict__ out) {
    __shared__ double red[kThreads];
    double s = 0.0;
    for (int i = threadIdx.x; i < nb; i += kThreads) s += part[i];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

struct Cgls {
    cudaStream_t s;
    int sms;
    DBuf<double> part, scal, seg;
    unsigned grid(int64_t n) const {
        return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, kThreads), 8 * sms));
    }
    double dot(int64_t n, const double *a, const double *b, int slot) {
        const unsigned g = std::min<unsigned>(grid(n), 1024);
        k_dot<<<g, kThreads, 0, s>>>(n, a, b, part.p);
        k_dot_final<<<1, kThreads, 0, s>>>((int)g, part.p, scal.p + slot);
        ERTGB_CUDA(cudaGetLastError());
        double h = 0.0;
        ERTGB_CUDA(cudaMemcpyAsync(&h, scal.p + slot, sizeof(double), cudaMemcpyDeviceToHost, s));
        ERTGB_CUDA(cudaStreamSynchronize(s));
        return h;
    }
};

}  // namespace

int cgls_solve(const void *J, int dtype, int64_t D, int64_t P, int64_t NC, const int32_t *c_rp, const int32_t *c_ci,
               const double *c_v, const int32_t *ct_rp, const int32_t *ct_ci, const double *ct_v, const double *dW,
               const double *b, double *x, const double *wc, const double *wm, const double *tm, const double *td,
               double lambda, const double *rough, int max_iter, double tol, int *iters, cudaStream_t s) {
    Cgls cg{s, 1};
    int dev = 0;
    ERTGB_CUDA(cudaGetDevice(&dev));
    cudaDeviceGetAttribute(&cg.sms, cudaDevAttrMultiProcessorCount, dev);
    cg.part.alloc(1024);
    cg.scal.alloc(8);
    cg.seg.alloc((size_t)kRowSeg * P);
    DBuf<double> cdx, z, p, r, q, tmpP, tmpD, tmpC, tmpC2, jt, ctc, dWtd;
    for (auto *v : {&cdx, &p, &r, &tmpP, &jt, &ctc}) v->alloc((size_t)P);
    for (auto *v : {&z, &q, &tmpD, &dWtd}) v->alloc((size_t)D);
    for (auto *v : {&tmpC, &tmpC2}) v->alloc((size_t)std::max<int64_t>(NC, 1));
    const unsigned gP = cg.grid(P), gD = cg.grid(D), gC = cg.grid(std::max<int64_t>(NC, 1));
    const dim3 gT((unsigned)ceil_div(P, kThreads), kRowSeg);
    const unsigned gJ = (unsigned)std::min<int64_t>(D, 16 * cg.sms);
    DBuf<float> x32, y32;
    const bool fast32 = dtype == 1 && (P & 3) == 0;
    if (fast32) {
        x32.alloc((size_t)P);
        y32.alloc((size_t)D);
    }
    const dim3 gT4((unsigned)ceil_div(P / 4, kThreads), kRowSeg);
    auto Jx = [&](const double *xin, const double *scale, double *yout) {
        if (dtype == 0) {
            k_jmul<double><<<gJ, kThreads, 0, s>>>(D, P, (const double *)J, xin, scale, yout);
        } else if (fast32) {
            k_to32<<<gP, kThreads, 0, s>>>(P, xin, x32.p);
            k_jmul32<<<gJ, kThreads, 0, s>>>(D, P, (const float *)J, x32.p, scale, yout);
        } else {
            k_jmul<float><<<gJ, kThreads, 0, s>>>(D, P, (const float *)J, xin, scale, yout);
        }
    };
    auto JTy = [&](const double *yin, const double *div, double *out) {
        if (dtype == 0) {
            k_jtmul<double><<<gT, kThreads, 0, s>>>(D, P, (const double *)J, yin, cg.seg.p);
        } else if (fast32) {
            k_to32<<<gD, kThreads, 0, s>>>(D, yin, y32.p);
            k_jtmul32<<<gT4, kThreads, 0, s>>>(D, P, (const float *)J, y32.p, cg.seg.p);
        } else {
            k_jtmul<float><<<gT, kThreads, 0, s>>>(D, P, (const float *)J, yin, cg.seg.p);
        }
        k_seg_sum<<<gP, kThreads, 0, s>>>(P, kRowSeg, cg.seg.p, div, out);
    };
    // C^T (C (wm x) wc^2) into out
    auto CtC = [&](const double *xin, double *out) {
        if (NC == 0) {
            ERTGB_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * P, s));
            return;
        }
        k_csr_mul<<<gC, kThreads, 0, s>>>(NC, c_rp, c_ci, c_v, xin, wm, 0, tmpC.p);
        k_mul4<<<gC, kThreads, 0, s>>>(NC, tmpC.p, wc, wc, nullptr, tmpC2.p);
        k_csr_mul<<<gP, kThreads, 0, s>>>(P, ct_rp, ct_ci, ct_v, tmpC2.p, nullptr, 0, out);
    };
    // dWtd = dW td; cdx = C^T (wc roughness) wm lambda
    k_mul4<<<gD, kThreads, 0, s>>>(D, dW, td, nullptr, nullptr, dWtd.p);
    if (NC > 0) {
        k_mul4<<<gC, kThreads, 0, s>>>(NC, wc, rough, nullptr, nullptr, tmpC.p);
        k_csr_mul<<<gP, kThreads, 0, s>>>(P, ct_rp, ct_ci, ct_v, tmpC.p, nullptr, 0, cdx.p);
        k_mul4<<<gP, kThreads, 0, s>>>(P, cdx.p, wm, nullptr, nullptr, cdx.p);
        k_scale<<<gP, kThreads, 0, s>>>(P, lambda, cdx.p);
    } else {
        ERTGB_CUDA(cudaMemsetAsync(cdx.p, 0, sizeof(double) * P, s));
    }
    // z = (b - (J (x/tm)) td) dW
    k_div<<<gP, kThreads, 0, s>>>(P, x, tm, tmpP.p);
    Jx(tmpP.p, td, tmpD.p);
    {
        DBuf<double> bmt;
        bmt.alloc((size_t)D);
        ERTGB_CUDA(cudaMemcpyAsync(bmt.p, b, sizeof(double) * D, cudaMemcpyDeviceToDevice, s));
        k_axpy<<<gD, kThreads, 0, s>>>(D, -1.0, tmpD.p, bmt.p);
        k_mul4<<<gD, kThreads, 0, s>>>(D, bmt.p, dW, nullptr, nullptr, z.p);
        ERTGB_CUDA(cudaStreamSynchronize(s));
    }
    // p = J^T(z dW td)/tm - C^T(wc^2 C(wm x)) wm lambda - cdx
    k_mul4<<<gD, kThreads, 0, s>>>(D, z.p, dWtd.p, nullptr, nullptr, tmpD.p);
    JTy(tmpD.p, tm, jt.p);
    CtC(x, ctc.p);
    k_rvec<<<gP, kThreads, 0, s>>>(P, jt.p, ctc.p, wm, lambda, cdx.p, p.p);
    // r = J^T(b dW^2 td)/tm - cdx   (only its norm sets the default accuracy)
    k_mul4<<<gD, kThreads, 0, s>>>(D, b, dW, dWtd.p, nullptr, tmpD.p);
    JTy(tmpD.p, tm, jt.p);
    ERTGB_CUDA(cudaMemsetAsync(ctc.p, 0, sizeof(double) * P, s));
    k_rvec<<<gP, kThreads, 0, s>>>(P, jt.p, ctc.p, wm, lambda, cdx.p, r.p);
    ERTGB_CUDA(cudaGetLastError());
    double accuracy = tol;
    if (accuracy < 0.0) accuracy = std::max(1e-12, 1e-8 * cg.dot(P, r.p, r.p, 0));
    ERTGB_CUDA(cudaMemcpyAsync(r.p, p.p, sizeof(double) * P, cudaMemcpyDeviceToDevice, s));
    double normR2 = cg.dot(P, r.p, r.p, 0);
    int count = 0;
    while (count < max_iter && normR2 > accuracy) {
        count++;
        k_div<<<gP, kThreads, 0, s>>>(P, p.p, tm, tmpP.p);
        Jx(tmpP.p, dWtd.p, q.p);  // q = (J (p/tm)) dW td
        double wcp2 = 0.0;
        if (NC > 0) {
            k_csr_mul<<<gC, kThreads, 0, s>>>(NC, c_rp, c_ci, c_v, p.p, wm, 1, tmpC.p);  // C (p wm), rounded
            k_mul4<<<gC, kThreads, 0, s>>>(NC, wc, tmpC.p, nullptr, nullptr, tmpC2.p);   // wcp
            wcp2 = cg.dot(NC, tmpC2.p, tmpC2.p, 1);
        }
        const double aQ = cg.dot(D, q.p, q.p, 2) + lambda * wcp2;
        const double alpha = normR2 / aQ;
        k_axpy<<<gP, kThreads, 0, s>>>(P, alpha, p.p, x);
        k_axpy<<<gD, kThreads, 0, s>>>(D, -alpha, q.p, z.p);
        k_mul4<<<gD, kThreads, 0, s>>>(D, z.p, dWtd.p, nullptr, nullptr, tmpD.p);
        JTy(tmpD.p, tm, jt.p);
        CtC(x, ctc.p);
        k_rvec<<<gP, kThreads, 0, s>>>(P, jt.p, ctc.p, wm, lambda, cdx.p, r.p);
        ERTGB_CUDA(cudaGetLastError());
        const double old = normR2;
        normR2 = cg.dot(P, r.p, r.p, 0);
        k_xpby<<<gP, kThreads, 0, s>>>(P, r.p, normR2 / old, p.p);
    }
    ERTGB_CUDA(cudaStreamSynchronize(s));
    if (iters) *iters = count;
    return std::isfinite(normR2) ? ERTGB_OK : ERTGB_NOT_CONVERGED;
}

}  // namespace ertgb
