// Complex resistivity (induced polarisation) on the GPU.
//
// With complex resistivities the reference's SR operator uses the total-
// potential formulation of DCMultiElectrodeModelling (calculateK_,
// core/src/bert/dcfemmodelling.cpp:1756-1929, the complex overload of
// calculateK at :1938-1942): per wavenumber the complex symmetric matrix
//   S* = sum_cells (1 / rho*_c) (K_c + k^2 M_c) + sum_mixed alpha_b / rho*_b M_b
// (dcfemmodelling.cpp:163-300 with complex attributes), a unit source at
// the current electrode's node (ElectrodeShapeNode::assembleRHS,
// core/src/bert/electrode.cpp:133-141), no singularity removal.  The
// potentials are summed over wavenumbers with their weights, collected at
// the electrodes (DataMap::collect / data, core/src/bert/datamap.cpp) and
// scaled by the geometric factors (dcfemmodelling.cpp:1103-1119).
//
// The reference factors every complex matrix (UMFPACK).  Here the nE x nK
// systems of one response are solved together by a block COCG (conjugate
// orthogonal CG: CG with the unconjugated bilinear form x^T y, valid for
// complex symmetric matrices; van der Vorst & Melissen 1990) with Jacobi
// preconditioning, FP64 throughout; a column stops when ||r||_2 <= rtol
// ||b||_2.  Dots are block partials reduced in a fixed order
// (deterministic).  The Jacobian is the reference's sensitivity
// (createSensitivityCol with complex potentials, J /= model^2 / k without
// conjugation, dcfemmodelling.cpp:1410-1431).
#include "ertgb_internal.cuh"
#include "reduce.cuh"

#include <algorithm>
#include <functional>

namespace ertgb {
namespace {

constexpr double kTolC = 1e-12;  // TOLERANCE of the reference (gimli.h)
constexpr int kRowsC = 8;        // rows per block in the vector kernels
constexpr int kPartC = 608;      // block partial rows of the column reductions
constexpr int kGraphItersC = 16; // iterations per CUDA graph launch

// per-column scalars (x Rpad)
enum CCol { C_RHO_RE = 0, C_RHO_IM, C_ALPHA_RE, C_ALPHA_IM, C_BETA_RE, C_BETA_IM, C_BB, C_RR, C_BEST, C_STALLS,
            C_NCOL };

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
// a / b (Smith's algorithm, scaled by the larger component of b)
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, d = b.x + b.y * r;
        return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
    }
    const double r = b.x / b.y, d = b.x * r + b.y;
    return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}

// sigma = 1 / rho* per cell; cells with |rho*| below the tolerance or not
// finite are counted (the caller rejects the model)
__global__ void k_sigma(int64_t C, const double *__restrict__ re, const double *__restrict__ im,
                        double2 *__restrict__ sigma, int32_t *__restrict__ bad) {
    for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < C; c += (int64_t)gridDim.x * blockDim.x) {
        const double2 z = make_double2(re[c], im[c]);
        const double a = hypot(z.x, z.y);
        if (!(a > kTolC) || !isfinite(a)) {
            atomicAdd(bad, 1);
            sigma[c] = make_double2(0.0, 0.0);
        } else {
            sigma[c] = cdiv(make_double2(1.0, 0.0), z);
        }
    }
}

// complex matrices of every wavenumber on the per-slot contribution lists
__global__ void k_assemble_c(int64_t nnz, const int32_t *__restrict__ cptr, const int32_t *__restrict__ centry,
                             const double *__restrict__ K, const double *__restrict__ M,
                             const double *__restrict__ bmass, const double *__restrict__ alpha,
                             const int32_t *__restrict__ bcell, const double2 *__restrict__ sigma,
                             const double *__restrict__ kv, int nv2, int nvb2, int64_t C, int64_t B,
                             double2 *__restrict__ vals) {
    const int ki = blockIdx.y;
    const double k = kv[ki];
    const double kk = k * k;
    const int64_t cbase = C * nv2;
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nnz; s += (int64_t)gridDim.x * blockDim.x) {
        double2 acc = make_double2(0.0, 0.0);
        const int32_t q1 = cptr[s + 1];
        for (int32_t q = cptr[s]; q < q1; q++) {
            const int64_t e = centry[q];
            if (e < cbase) {
                const double se = (k > 0.0) ? M[e] * kk + K[e] : K[e];
                acc = cadd(acc, cscale(sigma[e / nv2], se));
            } else {
                const int64_t eb = e - cbase;
                const int64_t b = eb / nvb2;
                acc = cadd(acc, cscale(sigma[bcell[b]], alpha[(int64_t)ki * B + b] * bmass[eb]));
            }
        }
        vals[(int64_t)ki * nnz + s] = acc;
    }
}

__global__ void k_dinv_c(int64_t n, int nK, int64_t nnz, const int32_t *__restrict__ diag,
                         const double2 *__restrict__ vals, double2 *__restrict__ dinv) {
    const int64_t total = n * nK;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ki = t / n, r = t - ki * n;
        dinv[t] = cdiv(make_double2(1.0, 0.0), vals[ki * nnz + diag[r]]);
    }
}

// unit sources: r[enode(e)][t] = 1 for column t = k nE + e < R
__global__ void k_sources_c(int nE, int64_t R, int64_t Rpad, const int32_t *__restrict__ enode,
                            double2 *__restrict__ r) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < R) r[(int64_t)enode[t % nE] * Rpad + t] = make_double2(1.0, 0.0);
}

// block partials of three column sums over the block's rows, reduced over
// the block's row lanes in a fixed order
__device__ __forceinline__ void block_partials3(double a, double b, double c, double *pa, double *pb, double *pc,
                                                int64_t Rpad, int64_t t) {
    __shared__ double sa[kRowsC][32], sb[kRowsC][32], sc[kRowsC][32];
    sa[threadIdx.y][threadIdx.x] = a;
    sb[threadIdx.y][threadIdx.x] = b;
    sc[threadIdx.y][threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.y == 0) {
        double s1 = 0.0, s2 = 0.0, s3 = 0.0;
        for (int w = 0; w < kRowsC; w++) {
            s1 += sa[w][threadIdx.x];
            s2 += sb[w][threadIdx.x];
            s3 += sc[w][threadIdx.x];
        }
        const int64_t o = (int64_t)blockIdx.y * Rpad + t;
        pa[o] = s1;
        if (pb) pb[o] = s2;
        if (pc) pc[o] = s3;
    }
}

// z = D^-1 r; with SETP also p = z (on the columns selected by ``sel``,
// all when null) else on the active columns.  Partials of r^T z (complex)
// and r^H r.
template <bool SETP>
__global__ void k_precond_c(int64_t n, int nE, int64_t R, int64_t Rpad, const double2 *__restrict__ dinv,
                            const int32_t *__restrict__ sel, const double2 *__restrict__ r,
                            double2 *__restrict__ z, double2 *__restrict__ p, double *__restrict__ p_re,
                            double *__restrict__ p_im, double *__restrict__ p_rr) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const bool act = t < R && (SETP ? (!sel || sel[t]) : sel[t] != 0);
    const double2 *dk = dinv + (t < R ? t / nE : 0) * n;
    double a = 0.0, b = 0.0, c = 0.0;
    if (act) {
        for (int64_t row = (int64_t)blockIdx.y * kRowsC + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRowsC) {
            const int64_t i = row * Rpad + t;
            const double2 rv = r[i];
            const double2 zv = cmul(dk[row], rv);
            z[i] = zv;
            if (SETP) p[i] = zv;
            const double2 rz = cmul(rv, zv);
            a += rz.x;
            b += rz.y;
            c += rv.x * rv.x + rv.y * rv.y;
        }
    }
    block_partials3(a, b, c, p_re, p_im, p_rr, Rpad, t);
}

// q = A p per column's wavenumber, partials of p^T q
__global__ void k_spmm_c(int64_t n, int64_t nnz, int nE, int64_t R, int64_t Rpad, const int32_t *__restrict__ rowptr,
                         const int32_t *__restrict__ colidx, const double2 *__restrict__ vals,
                         const int32_t *__restrict__ active, const double2 *__restrict__ p, double2 *__restrict__ q,
                         double *__restrict__ p_re, double *__restrict__ p_im) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const bool act = t < R && active[t];
    const double2 *vk = vals + (t < R ? t / nE : 0) * nnz;
    double a = 0.0, b = 0.0;
    if (act) {
        for (int64_t row = (int64_t)blockIdx.y * kRowsC + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRowsC) {
            double2 acc = make_double2(0.0, 0.0);
            const int32_t s1 = rowptr[row + 1];
            for (int32_t s = rowptr[row]; s < s1; s++)
                acc = cadd(acc, cmul(vk[s], p[(int64_t)colidx[s] * Rpad + t]));
            const int64_t i = row * Rpad + t;
            q[i] = acc;
            const double2 pq = cmul(p[i], acc);
            a += pq.x;
            b += pq.y;
        }
    }
    block_partials3(a, b, 0.0, p_re, p_im, nullptr, Rpad, t);
}

// x += alpha p, r -= alpha q on active columns
__global__ void k_update_xr_c(int64_t n, int64_t Rpad, const double *__restrict__ col,
                              const int32_t *__restrict__ active, double2 *__restrict__ x, double2 *__restrict__ r,
                              const double2 *__restrict__ p, const double2 *__restrict__ q) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (!active[t]) return;
    const double2 al = make_double2(col[C_ALPHA_RE * Rpad + t], col[C_ALPHA_IM * Rpad + t]);
    for (int64_t row = (int64_t)blockIdx.y * kRowsC + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRowsC) {
        const int64_t i = row * Rpad + t;
        x[i] = cadd(x[i], cmul(al, p[i]));
        r[i] = csub(r[i], cmul(al, q[i]));
    }
}

// p = z + beta p on active columns
__global__ void k_update_p_c(int64_t n, int64_t Rpad, const double *__restrict__ col,
                             const int32_t *__restrict__ active, const double2 *__restrict__ z,
                             double2 *__restrict__ p) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (!active[t]) return;
    const double2 be = make_double2(col[C_BETA_RE * Rpad + t], col[C_BETA_IM * Rpad + t]);
    for (int64_t row = (int64_t)blockIdx.y * kRowsC + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRowsC) {
        const int64_t i = row * Rpad + t;
        p[i] = cadd(z[i], cmul(be, p[i]));
    }
}

// initial column scalars: rho = r^T z, bb = rr = ||b||^2; active where b != 0
// initial column scalars: rho = r^T z, rr = ||r||^2, bb = ||b||^2 = 1 (unit
// sources); active where the residual is nonzero (with mask: and mask[t],
// a warm start of the selected columns keeping their iteration counts)
__global__ void k_finish_init_c(int64_t Rpad, int64_t R, int NB, const double *__restrict__ p_re,
                                const double *__restrict__ p_im, const double *__restrict__ p_rr,
                                double *__restrict__ col, int32_t *__restrict__ active, int32_t *__restrict__ iters,
                                int32_t *__restrict__ nactive, const int32_t *__restrict__ mask) {
    __shared__ double ra[32][33], rb[32][33], rc[32][33];
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const double re = col_sum(p_re, NB, Rpad, t, ra);
    const double im = col_sum(p_im, NB, Rpad, t, rb);
    const double rr = col_sum(p_rr, NB, Rpad, t, rc);
    if (threadIdx.y != 0) return;
    if (mask && !mask[t]) {
        active[t] = 0;
        return;
    }
    col[C_RHO_RE * Rpad + t] = re;
    col[C_RHO_IM * Rpad + t] = im;
    col[C_BB * Rpad + t] = t < R ? 1.0 : 0.0;
    col[C_RR * Rpad + t] = rr;
    col[C_BEST * Rpad + t] = rr;
    col[C_STALLS * Rpad + t] = 0.0;
    const int a = (t < R && rr > 0.0) ? 1 : 0;
    active[t] = a;
    if (!mask) iters[t] = 0;
    if (a) atomicAdd(nactive, 1);
}

// alpha = rho / (p^T q); a column whose p^T q vanishes (breakdown) stops
__global__ void k_finish_alpha_c(int64_t Rpad, int NB, const double *__restrict__ p_re,
                                 const double *__restrict__ p_im, double *__restrict__ col,
                                 int32_t *__restrict__ active, int32_t *__restrict__ nactive) {
    __shared__ double ra[32][33], rb[32][33];
    if (blockIdx.x == 0 && threadIdx.x == 0 && threadIdx.y == 0) *nactive = 0;
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const double2 pq = make_double2(col_sum(p_re, NB, Rpad, t, ra), col_sum(p_im, NB, Rpad, t, rb));
    if (threadIdx.y != 0 || !active[t]) return;
    const double2 rho = make_double2(col[C_RHO_RE * Rpad + t], col[C_RHO_IM * Rpad + t]);
    double2 al = make_double2(0.0, 0.0);
    if (hypot(pq.x, pq.y) > 0.0) al = cdiv(rho, pq);
    if (!isfinite(al.x) || !isfinite(al.y)) al = make_double2(0.0, 0.0);
    col[C_ALPHA_RE * Rpad + t] = al.x;
    col[C_ALPHA_IM * Rpad + t] = al.y;
}

// beta = rho_new / rho, convergence ||r||^2 <= rtol^2 ||b||^2
__global__ void k_finish_beta_c(int64_t Rpad, int NB, double rtol2, const double *__restrict__ p_re,
                                const double *__restrict__ p_im, const double *__restrict__ p_rr,
                                double *__restrict__ col, int32_t *__restrict__ active, int32_t *__restrict__ iters,
                                int32_t *__restrict__ nactive) {
    __shared__ double ra[32][33], rb[32][33], rc[32][33];
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const double2 rz = make_double2(col_sum(p_re, NB, Rpad, t, ra), col_sum(p_im, NB, Rpad, t, rb));
    const double rr = col_sum(p_rr, NB, Rpad, t, rc);
    if (threadIdx.y != 0 || !active[t]) return;
    iters[t] += 1;
    col[C_RR * Rpad + t] = rr;
    const double2 rho = make_double2(col[C_RHO_RE * Rpad + t], col[C_RHO_IM * Rpad + t]);
    double2 be = make_double2(0.0, 0.0);
    if (hypot(rho.x, rho.y) > 0.0) be = cdiv(rz, rho);
    col[C_BETA_RE * Rpad + t] = be.x;
    col[C_BETA_IM * Rpad + t] = be.y;
    col[C_RHO_RE * Rpad + t] = rz.x;
    col[C_RHO_IM * Rpad + t] = rz.y;
    if (!(rr > rtol2 * col[C_BB * Rpad + t])) {
        active[t] = 0;  // converged (or not finite: stops too, reported by the residual check)
    } else {
        atomicAdd(nactive, 1);
    }
}

// U[e][f] = sum_k w_k x[enode(f)][k nE + e]
__global__ void k_collect_c(int nE, int nK, int64_t Rpad, const int32_t *__restrict__ enode,
                            const double *__restrict__ w, const double2 *__restrict__ x, double2 *__restrict__ U) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)nE * nE) return;
    const int e = (int)(i / nE), f = (int)(i % nE);
    double2 acc = make_double2(0.0, 0.0);
    for (int k = 0; k < nK; k++) acc = cadd(acc, cscale(x[(int64_t)enode[f] * Rpad + (int64_t)k * nE + e], w[k]));
    U[i] = acc;
}

// k * ((U[a][m] - U[a][n]) - (U[b][m] - U[b][n])), -1 = electrode at infinity
__global__ void k_response_c(int64_t D, int nE, const int32_t *__restrict__ abmn, const double *__restrict__ kfac,
                             const double2 *__restrict__ U, double *__restrict__ out_re, double *__restrict__ out_im) {
    const int64_t d = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= D) return;
    const int a = abmn[4 * d], b = abmn[4 * d + 1], m = abmn[4 * d + 2], n = abmn[4 * d + 3];
    auto u = [&](int i, int j) {
        return (i != -1 && j != -1) ? U[(int64_t)i * nE + j] : make_double2(0.0, 0.0);
    };
    const double2 v = csub(csub(u(a, m), u(a, n)), csub(u(b, m), u(b, n)));
    out_re[d] = v.x * kfac[d];
    out_im[d] = v.y * kfac[d];
}

unsigned grid1c(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 32)); }

}  // namespace

namespace {

// Complex Jacobian: block per parameter (its cells in ascending order, so the
// sum is deterministic), threads over data; for every cell and wavenumber
// J[d, p] += w_k (u_a - u_b)^T (K_c + k^2 M_c) (u_m - u_n) with the local
// complex potentials, then J[d, p] *= k_d / model_p^2 (complex, no
// conjugation) when the model has one value per parameter.
__global__ void k_jacobian_c(int64_t D, int64_t P, int nE, int nK, int64_t Rpad, int nv,
                             const int32_t *__restrict__ abmn, const double *__restrict__ kfac,
                             const int32_t *__restrict__ pcell_ptr, const int32_t *__restrict__ pcell,
                             const int32_t *__restrict__ cells, const double *__restrict__ K,
                             const double *__restrict__ M, const double *__restrict__ kv,
                             const double *__restrict__ w, const double2 *__restrict__ x,
                             const double *__restrict__ m_re, const double *__restrict__ m_im,
                             double2 *__restrict__ J) {
    __shared__ double Se[100];  // nv x nv <= 10 x 10
    __shared__ int32_t nodes[10];
    const int64_t p = blockIdx.x;
    const int64_t d = (int64_t)blockIdx.y * blockDim.x + threadIdx.x;
    int a = -1, b = -1, m = -1, n = -1;
    if (d < D) {
        a = abmn[4 * d];
        b = abmn[4 * d + 1];
        m = abmn[4 * d + 2];
        n = abmn[4 * d + 3];
    }
    double2 acc = make_double2(0.0, 0.0);
    const int nv2 = nv * nv;
    for (int32_t q = pcell_ptr[p]; q < pcell_ptr[p + 1]; q++) {
        const int64_t c = pcell[q];
        for (int ki = 0; ki < nK; ki++) {
            const double kk = kv[ki] * kv[ki];
            __syncthreads();
            for (int i = threadIdx.x; i < nv2; i += blockDim.x)
                Se[i] = kv[ki] > 0.0 ? M[c * nv2 + i] * kk + K[c * nv2 + i] : K[c * nv2 + i];
            for (int i = threadIdx.x; i < nv; i += blockDim.x) nodes[i] = cells[c * nv + i];
            __syncthreads();
            if (d >= D) continue;
            const int64_t col0 = (int64_t)ki * nE;
            double2 dab[10], dmn[10];
            for (int i = 0; i < nv; i++) {
                const double2 *xr = x + (int64_t)nodes[i] * Rpad + col0;
                const double2 z0 = make_double2(0.0, 0.0);
                dab[i] = csub(a >= 0 ? xr[a] : z0, b >= 0 ? xr[b] : z0);
                dmn[i] = csub(m >= 0 ? xr[m] : z0, n >= 0 ? xr[n] : z0);
            }
            double2 s = make_double2(0.0, 0.0);
            for (int i = 0; i < nv; i++) {
                double2 sv = make_double2(0.0, 0.0);
                for (int j = 0; j < nv; j++) sv = cadd(sv, cscale(dmn[j], Se[i * nv + j]));
                s = cadd(s, cmul(dab[i], sv));
            }
            acc = cadd(acc, cscale(s, w[ki]));
        }
    }
    if (d >= D) return;
    if (m_re) {
        const double2 mp = make_double2(m_re[p], m_im[p]);
        acc = cdiv(cscale(acc, kfac[d]), cmul(mp, mp));
    }
    J[d * P + p] = acc;
}

}  // namespace

namespace {

// ---- mixed precision: FP32 complex recurrence, FP64 reliable updates -------

__device__ __forceinline__ float2 fmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 fadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 fsub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

__global__ void k_to_f32_c(int64_t n, const double2 *__restrict__ a, float2 *__restrict__ b) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = make_float2((float)a[i].x, (float)a[i].y);
}

// r = b - A x in FP64 (b: unit sources) on the columns t < R with mask[t]
// (all when mask is null).  F32: also r32 = r, z32 = D^-1 r32 and partials
// of r^T z (FP32 values) and ||r||^2 (FP64); else r64 = r.
template <bool F32>
__global__ void k_resid_c(int64_t n, int64_t nnz, int nE, int64_t R, int64_t Rpad, const int32_t *__restrict__ rowptr,
                          const int32_t *__restrict__ colidx, const double2 *__restrict__ vals,
                          const int32_t *__restrict__ enode, const int32_t *__restrict__ mask,
                          const double2 *__restrict__ x, double2 *__restrict__ r64, const float2 *__restrict__ dinv32,
                          float2 *__restrict__ r32, float2 *__restrict__ z32, double *__restrict__ p_re,
                          double *__restrict__ p_im, double *__restrict__ p_rr) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const bool act = t < R && (!mask || mask[t]);
    const int64_t ki = t < R ? t / nE : 0;
    const double2 *vk = vals + ki * nnz;
    const float2 *dk = F32 ? dinv32 + ki * n : nullptr;
    const int32_t src = t < R ? enode[t % nE] : -1;
    double a = 0.0, b = 0.0, c = 0.0;
    if (act) {
        for (int64_t row = (int64_t)blockIdx.y * kRowsC + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRowsC) {
            double2 acc = make_double2(row == src ? 1.0 : 0.0, 0.0);
            const int32_t s1 = rowptr[row + 1];
            for (int32_t s = rowptr[row]; s < s1; s++) acc = csub(acc, cmul(vk[s], x[(int64_t)colidx[s] * Rpad + t]));
            const int64_t i = row * Rpad + t;
            c += acc.x * acc.x + acc.y * acc.y;
            if (F32) {
                const float2 rv = make_float2((float)acc.x, (float)acc.y);
                const float2 zv = fmul(dk[row], rv);
                r32[i] = rv;
                z32[i] = zv;
                const float2 rz = fmul(rv, zv);
                a += rz.x;
                b += rz.y;
            } else {
                r64[i] = acc;
            }
        }
    }
    block_partials3(a, b, c, p_re, p_im, p_rr, Rpad, t);
}

// q = A p in FP32, partials of p^T q
__global__ void k_spmm_c32(int64_t n, int64_t nnz, int nE, int64_t R, int64_t Rpad, const int32_t *__restrict__ rowptr,
                           const int32_t *__restrict__ colidx, const float2 *__restrict__ vals,
                           const int32_t *__restrict__ active, const float2 *__restrict__ p, float2 *__restrict__ q,
                           double *__restrict__ p_re, double *__restrict__ p_im) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const bool act = t < R && active[t];
    const float2 *vk = vals + (t < R ? t / nE : 0) * nnz;
    float a = 0.f, b = 0.f;
    if (act) {
        for (int64_t row = (int64_t)blockIdx.y * kRowsC + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRowsC) {
            float2 acc = make_float2(0.f, 0.f);
            const int32_t s1 = rowptr[row + 1];
            for (int32_t s = rowptr[row]; s < s1; s++) acc = fadd(acc, fmul(vk[s], p[(int64_t)colidx[s] * Rpad + t]));
            const int64_t i = row * Rpad + t;
            q[i] = acc;
            const float2 pq = fmul(p[i], acc);
            a += pq.x;
            b += pq.y;
        }
    }
    block_partials3(a, b, 0.0, p_re, p_im, nullptr, Rpad, t);
}

// q = A p for one wavenumber (3-D): an 8-lane group per row, every lane a
// float4 = two complex columns per chunk, CH chunks of 16 columns (Rpad =
// 16 CH), rows of a block contiguous; column dots p^T q per lane, summed over
// the block's groups in FP64 in a fixed order.
constexpr int kCqThreads = 256;
constexpr int kCqGroups = kCqThreads / 8;

template <int CH>
__global__ void __launch_bounds__(kCqThreads, 2) k_spmm_c32q(int64_t n, int64_t Rpad, const int32_t *__restrict__ rowptr,
                                                              const int32_t *__restrict__ colidx,
                                                              const float2 *__restrict__ vals,
                                                              const float2 *__restrict__ p, float2 *__restrict__ q,
                                                              double *__restrict__ p_re, double *__restrict__ p_im) {
    __shared__ float red[kCqGroups][32 * CH + 1];
    const int l8 = threadIdx.x & 7, g = threadIdx.x >> 3;
    const int64_t per_block = (n + gridDim.x - 1) / gridDim.x;
    const int64_t r_begin = (int64_t)blockIdx.x * per_block;
    const int64_t r_end = min(n, r_begin + per_block);
    float4 dot[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) dot[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int64_t row = r_begin + g; row < r_end; row += kCqGroups) {
        float4 acc[CH];
#pragma unroll
        for (int j = 0; j < CH; j++) acc[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        const int32_t s1 = rowptr[row + 1];
#pragma unroll 2
        for (int32_t s = rowptr[row]; s < s1; s++) {
            const int64_t col = colidx[s];
            const float2 v = vals[s];
            const float4 *pc = reinterpret_cast<const float4 *>(p + col * Rpad) + l8;
#pragma unroll
            for (int j = 0; j < CH; j++) {
                const float4 x = __ldg(pc + 8 * j);
                acc[j].x = fmaf(v.x, x.x, fmaf(-v.y, x.y, acc[j].x));
                acc[j].y = fmaf(v.x, x.y, fmaf(v.y, x.x, acc[j].y));
                acc[j].z = fmaf(v.x, x.z, fmaf(-v.y, x.w, acc[j].z));
                acc[j].w = fmaf(v.x, x.w, fmaf(v.y, x.z, acc[j].w));
            }
        }
        float4 *qr = reinterpret_cast<float4 *>(q + row * Rpad) + l8;
        const float4 *pr = reinterpret_cast<const float4 *>(p + row * Rpad) + l8;
#pragma unroll
        for (int j = 0; j < CH; j++) {
            qr[8 * j] = acc[j];
            const float4 d = pr[8 * j];
            dot[j].x += d.x * acc[j].x - d.y * acc[j].y;
            dot[j].y += d.x * acc[j].y + d.y * acc[j].x;
            dot[j].z += d.z * acc[j].z - d.w * acc[j].w;
            dot[j].w += d.z * acc[j].w + d.w * acc[j].z;
        }
    }
    // lane l8, chunk j holds columns 16 j + 2 l8 and + 1 as (re, im, re, im)
#pragma unroll
    for (int j = 0; j < CH; j++) {
        const int c = 4 * (8 * j + l8);
        red[g][c] = dot[j].x;
        red[g][c + 1] = dot[j].y;
        red[g][c + 2] = dot[j].z;
        red[g][c + 3] = dot[j].w;
    }
    __syncthreads();
    for (int c = threadIdx.x; c < 32 * CH; c += kCqThreads) {
        double sum = 0.0;
#pragma unroll 8
        for (int gg = 0; gg < kCqGroups; gg++) sum += (double)red[gg][c];
        const int64_t t = c >> 1;  // column
        if (c & 1) p_im[(int64_t)blockIdx.x * Rpad + t] = sum;
        else p_re[(int64_t)blockIdx.x * Rpad + t] = sum;
    }
}

// alpha = rho / (p^T q), one warp per column (warp_col_sum)
__global__ void k_finish_alpha_cw(int64_t Rpad, int NB, const double *__restrict__ p_re,
                                  const double *__restrict__ p_im, double *__restrict__ col,
                                  const int32_t *__restrict__ active, int32_t *__restrict__ nactive) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *nactive = 0;
    const int64_t t = (int64_t)blockIdx.x * kFinWarps + (threadIdx.x >> 5);
    if (t >= Rpad) return;
    const double2 pq = make_double2(warp_col_sum(p_re, NB, Rpad, t), warp_col_sum(p_im, NB, Rpad, t));
    if ((threadIdx.x & 31) != 0 || !active[t]) return;
    const double2 rho = make_double2(col[C_RHO_RE * Rpad + t], col[C_RHO_IM * Rpad + t]);
    double2 al = make_double2(0.0, 0.0);
    if (hypot(pq.x, pq.y) > 0.0) al = cdiv(rho, pq);
    if (!isfinite(al.x) || !isfinite(al.y)) al = make_double2(0.0, 0.0);
    col[C_ALPHA_RE * Rpad + t] = al.x;
    col[C_ALPHA_IM * Rpad + t] = al.y;
}

// recursive beta (mixed), one warp per column
__global__ void k_finish_beta_mcw(int64_t Rpad, int NB, const double *__restrict__ p_re,
                                  const double *__restrict__ p_im, double *__restrict__ col,
                                  const int32_t *__restrict__ active, int32_t *__restrict__ iters) {
    const int64_t t = (int64_t)blockIdx.x * kFinWarps + (threadIdx.x >> 5);
    if (t >= Rpad) return;
    const double2 rz = make_double2(warp_col_sum(p_re, NB, Rpad, t), warp_col_sum(p_im, NB, Rpad, t));
    if ((threadIdx.x & 31) != 0 || !active[t]) return;
    iters[t] += 1;
    const double2 rho = make_double2(col[C_RHO_RE * Rpad + t], col[C_RHO_IM * Rpad + t]);
    double2 be = make_double2(0.0, 0.0);
    if (hypot(rho.x, rho.y) > 0.0) be = cdiv(rz, rho);
    if (!isfinite(be.x) || !isfinite(be.y)) be = make_double2(0.0, 0.0);
    col[C_BETA_RE * Rpad + t] = be.x;
    col[C_BETA_IM * Rpad + t] = be.y;
    col[C_RHO_RE * Rpad + t] = rz.x;
    col[C_RHO_IM * Rpad + t] = rz.y;
}

// y += alpha p, r -= alpha q, z = D^-1 r; partials of r^T z and ||r||^2
__global__ void k_update_yrz_c32(int64_t n, int nE, int64_t R, int64_t Rpad, const double *__restrict__ col,
                                 const int32_t *__restrict__ active, const float2 *__restrict__ dinv32,
                                 float2 *__restrict__ y, float2 *__restrict__ r, float2 *__restrict__ z,
                                 const float2 *__restrict__ p, const float2 *__restrict__ q, double *__restrict__ p_re,
                                 double *__restrict__ p_im, double *__restrict__ p_rr) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const bool act = t < R && active[t];
    const float2 al = make_float2((float)col[C_ALPHA_RE * Rpad + t], (float)col[C_ALPHA_IM * Rpad + t]);
    const float2 *dk = dinv32 + (t < R ? t / nE : 0) * n;
    float a = 0.f, b = 0.f, c = 0.f;
    if (act) {
        for (int64_t row = (int64_t)blockIdx.y * kRowsC + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRowsC) {
            const int64_t i = row * Rpad + t;
            y[i] = fadd(y[i], fmul(al, p[i]));
            const float2 rv = fsub(r[i], fmul(al, q[i]));
            r[i] = rv;
            const float2 zv = fmul(dk[row], rv);
            z[i] = zv;
            const float2 rz = fmul(rv, zv);
            a += rz.x;
            b += rz.y;
            c += rv.x * rv.x + rv.y * rv.y;
        }
    }
    block_partials3(a, b, c, p_re, p_im, p_rr, Rpad, t);
}

__global__ void k_update_p_c32(int64_t n, int64_t Rpad, const double *__restrict__ col,
                               const int32_t *__restrict__ active, const float2 *__restrict__ z,
                               float2 *__restrict__ p) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (!active[t]) return;
    const float2 be = make_float2((float)col[C_BETA_RE * Rpad + t], (float)col[C_BETA_IM * Rpad + t]);
    for (int64_t row = (int64_t)blockIdx.y * kRowsC + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRowsC) {
        const int64_t i = row * Rpad + t;
        p[i] = fadd(z[i], fmul(be, p[i]));
    }
}

// reliable update, part 1: x += y, y = 0 on active columns; counter reset
__global__ void k_accum_c(int64_t n, int64_t Rpad, const int32_t *__restrict__ active, double2 *__restrict__ x,
                          float2 *__restrict__ y, int32_t *__restrict__ nactive) {
    if (blockIdx.x == 0 && blockIdx.y == 0 && threadIdx.x == 0 && threadIdx.y == 0) *nactive = 0;
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (!active[t]) return;
    for (int64_t row = (int64_t)blockIdx.y * kRowsC + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRowsC) {
        const int64_t i = row * Rpad + t;
        const float2 v = y[i];
        x[i] = make_double2(x[i].x + (double)v.x, x[i].y + (double)v.y);
        y[i] = make_float2(0.f, 0.f);
    }
}

// reliable update, part 3: convergence on the FP64 true residual, rho of the
// restarted residual, stall detection as in the real mixed solver: no 10 %
// improvement of the best residual over four intervals, or divergence
// (above 4 ||b||^2, or not finite), hands the column to the FP64 solver
// (stalled 1: warm start from its x; 2: from zero).
__global__ void k_finish_ru_c(int64_t Rpad, int NB, double rtol2, const double *__restrict__ p_re,
                              const double *__restrict__ p_im, const double *__restrict__ p_rr,
                              double *__restrict__ col, int32_t *__restrict__ active, int32_t *__restrict__ stalled,
                              int32_t *__restrict__ nactive, int32_t *__restrict__ nstalled) {
    __shared__ double ra[32][33], rb[32][33], rc[32][33];
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const double2 rz = make_double2(col_sum(p_re, NB, Rpad, t, ra), col_sum(p_im, NB, Rpad, t, rb));
    const double rr = col_sum(p_rr, NB, Rpad, t, rc);
    if (threadIdx.y != 0 || !active[t]) return;
    const double bb = col[C_BB * Rpad + t];
    col[C_RR * Rpad + t] = rr;
    col[C_RHO_RE * Rpad + t] = rz.x;
    col[C_RHO_IM * Rpad + t] = rz.y;
    if (rr <= rtol2 * bb) {
        active[t] = 0;
        return;
    }
    if (!(rr <= 4.0 * bb) || !isfinite(rz.x) || !isfinite(rz.y)) {
        active[t] = 0;
        stalled[t] = 2;
        atomicAdd(nstalled, 1);
        return;
    }
    double stalls = col[C_STALLS * Rpad + t];
    if (rr < 0.81 * col[C_BEST * Rpad + t]) {
        col[C_BEST * Rpad + t] = rr;
        stalls = 0.0;
    } else {
        stalls += 1.0;
    }
    col[C_STALLS * Rpad + t] = stalls;
    if (stalls >= 4.0) {
        active[t] = 0;
        stalled[t] = 1;
        atomicAdd(nstalled, 1);
        return;
    }
    atomicAdd(nactive, 1);
}

// stalled columns restarting from zero: x = 0 there
__global__ void k_zero_restart_c(int64_t n, int64_t Rpad, const int32_t *__restrict__ stalled,
                                 double2 *__restrict__ x) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    if (stalled[t] != 2) return;
    for (int64_t row = (int64_t)blockIdx.y * kRowsC + threadIdx.y; row < n; row += (int64_t)gridDim.y * kRowsC)
        x[row * Rpad + t] = make_double2(0.0, 0.0);
}

}  // namespace

namespace {

struct CxLaunch {
    int64_t n, nnz, R, Rpad;
    int NB;
    dim3 vb, vg, fb, fg;
};

void run_graph_loop(Context &c, cudaStream_t s, const std::function<void()> &body, int32_t *nactive, int launches,
                    const std::function<void()> &after, int *status) {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    try {
        ERTGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        body();
        ERTGB_CUDA(cudaStreamEndCapture(s, &g));
        ERTGB_CUDA(cudaGraphInstantiate(&ge, g, 0));
        int32_t h_active = 0;
        ERTGB_CUDA(cudaMemcpyAsync(&h_active, nactive, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        ERTGB_CUDA(cudaStreamSynchronize(s));
        int done = 0;
        while (h_active > 0) {
            if (done >= c.max_iter) {
                *status = ERTGB_NOT_CONVERGED;
                break;
            }
            for (int u = 0; u < launches; u++) ERTGB_CUDA(cudaGraphLaunch(ge, s));
            done += launches * kGraphItersC;
            if (after) after();
            ERTGB_CUDA(cudaMemcpyAsync(&h_active, nactive, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
            ERTGB_CUDA(cudaStreamSynchronize(s));
        }
    } catch (...) {
        cudaGraph_t dummy = nullptr;
        cudaStreamEndCapture(s, &dummy);
        if (dummy) cudaGraphDestroy(dummy);
        if (ge) cudaGraphExecDestroy(ge);
        if (g) cudaGraphDestroy(g);
        throw;
    }
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
}

// FP64 block COCG; mask: warm start of the columns with mask[t] != 0 from x
int cocg_fp64(Context &c, const CxLaunch &L, cudaStream_t s, const int32_t *mask) {
    MeshData &m = c.mesh;
    ComplexState &x = c.cx;
    const int64_t n = L.n, nnz = L.nnz, R = L.R, Rpad = L.Rpad;
    const int NB = L.NB;
    double *pa = x.part.p, *pb = pa + (size_t)NB * Rpad, *pc = pb + (size_t)NB * Rpad;
    double *pd = pc + (size_t)NB * Rpad, *pe = pd + (size_t)NB * Rpad;
    int32_t *active = x.active.p, *iters = active + Rpad, *nactive = active + 2 * Rpad;
    if (!mask) ERTGB_CUDA(cudaMemsetAsync(x.x.p, 0, sizeof(double2) * n * Rpad, s));
    ERTGB_CUDA(cudaMemsetAsync(nactive, 0, sizeof(int32_t), s));
    k_resid_c<false><<<L.vg, L.vb, 0, s>>>(n, nnz, c.nE, R, Rpad, m.d_rowptr.p, m.d_colidx.p, x.S.p, c.d_enode.p, mask,
                                           x.x.p, x.r.p, nullptr, nullptr, nullptr, pa, pb, pc);
    k_precond_c<true><<<L.vg, L.vb, 0, s>>>(n, c.nE, R, Rpad, x.dinv.p, mask, x.r.p, x.z.p, x.p.p, pa, pb, pc);
    k_finish_init_c<<<L.fg, L.fb, 0, s>>>(Rpad, R, NB, pa, pb, pc, x.col.p, active, iters, nactive, mask);
    ERTGB_CUDA(cudaGetLastError());
    const double rtol2 = c.rtol * c.rtol;
    int status = ERTGB_OK;
    run_graph_loop(c, s, [&] {
        for (int it = 0; it < kGraphItersC; it++) {
            k_spmm_c<<<L.vg, L.vb, 0, s>>>(n, nnz, c.nE, R, Rpad, m.d_rowptr.p, m.d_colidx.p, x.S.p, active, x.p.p,
                                           x.q.p, pd, pe);
            k_finish_alpha_c<<<L.fg, L.fb, 0, s>>>(Rpad, NB, pd, pe, x.col.p, active, nactive);
            k_update_xr_c<<<L.vg, L.vb, 0, s>>>(n, Rpad, x.col.p, active, x.x.p, x.r.p, x.p.p, x.q.p);
            k_precond_c<false><<<L.vg, L.vb, 0, s>>>(n, c.nE, R, Rpad, x.dinv.p, active, x.r.p, x.z.p, nullptr, pa,
                                                     pb, pc);
            k_finish_beta_c<<<L.fg, L.fb, 0, s>>>(Rpad, NB, rtol2, pa, pb, pc, x.col.p, active, iters, nactive);
            k_update_p_c<<<L.vg, L.vb, 0, s>>>(n, Rpad, x.col.p, active, x.z.p, x.p.p);
        }
    }, nactive, 4, nullptr, &status);
    return status;
}

// mixed block COCG: FP32 recurrence (matrix, vectors), FP64 solution, FP64
// true residual every 4 x 16 iterations; returns the number of stalled columns
int cocg_mixed(Context &c, const CxLaunch &L, cudaStream_t s, int *status) {
    MeshData &m = c.mesh;
    ComplexState &x = c.cx;
    const int64_t n = L.n, nnz = L.nnz, R = L.R, Rpad = L.Rpad;
    const int NB = L.NB;
    double *pa = x.part.p, *pb = pa + (size_t)NB * Rpad, *pc = pb + (size_t)NB * Rpad;
    double *pd = pc + (size_t)NB * Rpad, *pe = pd + (size_t)NB * Rpad;
    int32_t *active = x.active.p, *iters = active + Rpad, *nactive = active + 2 * Rpad;
    int32_t *stalled = x.stalled.p, *nstalled = stalled + Rpad;
    x.S32.alloc((size_t)c.nK * nnz);
    x.dinv32.alloc((size_t)c.nK * n);
    for (DBuf<float2> *v : {&x.r32, &x.z32, &x.p32, &x.q32, &x.y32}) v->alloc((size_t)n * Rpad);
    k_to_f32_c<<<grid1c(c.nK * nnz), 256, 0, s>>>(c.nK * nnz, x.S.p, x.S32.p);
    k_to_f32_c<<<grid1c(c.nK * n), 256, 0, s>>>(c.nK * n, x.dinv.p, x.dinv32.p);
    ERTGB_CUDA(cudaMemsetAsync(x.x.p, 0, sizeof(double2) * n * Rpad, s));
    ERTGB_CUDA(cudaMemsetAsync(x.y32.p, 0, sizeof(float2) * n * Rpad, s));
    ERTGB_CUDA(cudaMemsetAsync(stalled, 0, sizeof(int32_t) * (Rpad + 1), s));
    ERTGB_CUDA(cudaMemsetAsync(nactive, 0, sizeof(int32_t), s));
    k_resid_c<true><<<L.vg, L.vb, 0, s>>>(n, nnz, c.nE, R, Rpad, m.d_rowptr.p, m.d_colidx.p, x.S.p, c.d_enode.p,
                                          nullptr, x.x.p, nullptr, x.dinv32.p, x.r32.p, x.z32.p, pa, pb, pc);
    ERTGB_CUDA(cudaMemcpyAsync(x.p32.p, x.z32.p, sizeof(float2) * n * Rpad, cudaMemcpyDeviceToDevice, s));
    k_finish_init_c<<<L.fg, L.fb, 0, s>>>(Rpad, R, NB, pa, pb, pc, x.col.p, active, iters, nactive, nullptr);
    ERTGB_CUDA(cudaGetLastError());
    const double rtol2 = c.rtol * c.rtol;
    // the reliable update as a second graph
    cudaGraph_t gru = nullptr;
    cudaGraphExec_t eru = nullptr;
    ERTGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    k_accum_c<<<L.vg, L.vb, 0, s>>>(n, Rpad, active, x.x.p, x.y32.p, nactive);
    k_resid_c<true><<<L.vg, L.vb, 0, s>>>(n, nnz, c.nE, R, Rpad, m.d_rowptr.p, m.d_colidx.p, x.S.p, c.d_enode.p, active,
                                          x.x.p, nullptr, x.dinv32.p, x.r32.p, x.z32.p, pa, pb, pc);
    k_finish_ru_c<<<L.fg, L.fb, 0, s>>>(Rpad, NB, rtol2, pa, pb, pc, x.col.p, active, stalled, nactive, nstalled);
    ERTGB_CUDA(cudaStreamEndCapture(s, &gru));
    ERTGB_CUDA(cudaGraphInstantiate(&eru, gru, 0));
    // one wavenumber and Rpad = 16 CH: the 8-lane-group operator (partials of NBq block rows)
    const int chq = c.nK == 1 ? (int)(Rpad / 16) : 0;
    const bool fastq = chq == 2 || chq == 4 || chq == 6 || chq == 8;
    const int NBq = fastq ? (int)std::min<int64_t>(ceil_div(n, kCqGroups), 304) : NB;
    const unsigned fwg = (unsigned)ceil_div(Rpad, kFinWarps);
    auto spmm = [&] {
        switch (fastq ? chq : 0) {
            case 2: k_spmm_c32q<2><<<NBq, kCqThreads, 0, s>>>(n, Rpad, m.d_rowptr.p, m.d_colidx.p, x.S32.p, x.p32.p,
                                                             x.q32.p, pd, pe); break;
            case 4: k_spmm_c32q<4><<<NBq, kCqThreads, 0, s>>>(n, Rpad, m.d_rowptr.p, m.d_colidx.p, x.S32.p, x.p32.p,
                                                             x.q32.p, pd, pe); break;
            case 6: k_spmm_c32q<6><<<NBq, kCqThreads, 0, s>>>(n, Rpad, m.d_rowptr.p, m.d_colidx.p, x.S32.p, x.p32.p,
                                                             x.q32.p, pd, pe); break;
            case 8: k_spmm_c32q<8><<<NBq, kCqThreads, 0, s>>>(n, Rpad, m.d_rowptr.p, m.d_colidx.p, x.S32.p, x.p32.p,
                                                             x.q32.p, pd, pe); break;
            default: k_spmm_c32<<<L.vg, L.vb, 0, s>>>(n, nnz, c.nE, R, Rpad, m.d_rowptr.p, m.d_colidx.p, x.S32.p,
                                                      active, x.p32.p, x.q32.p, pd, pe);
        }
    };
    try {
        run_graph_loop(c, s, [&] {
            for (int it = 0; it < kGraphItersC; it++) {
                spmm();
                k_finish_alpha_cw<<<fwg, 32 * kFinWarps, 0, s>>>(Rpad, NBq, pd, pe, x.col.p, active, nactive);
                k_update_yrz_c32<<<L.vg, L.vb, 0, s>>>(n, c.nE, R, Rpad, x.col.p, active, x.dinv32.p, x.y32.p,
                                                       x.r32.p, x.z32.p, x.p32.p, x.q32.p, pa, pb, pc);
                k_finish_beta_mcw<<<fwg, 32 * kFinWarps, 0, s>>>(Rpad, NB, pa, pb, x.col.p, active, iters);
                k_update_p_c32<<<L.vg, L.vb, 0, s>>>(n, Rpad, x.col.p, active, x.z32.p, x.p32.p);
            }
        }, nactive, 4, [&] { ERTGB_CUDA(cudaGraphLaunch(eru, s)); }, status);
    } catch (...) {
        cudaGraphExecDestroy(eru);
        cudaGraphDestroy(gru);
        throw;
    }
    cudaGraphExecDestroy(eru);
    cudaGraphDestroy(gru);
    if (*status == ERTGB_NOT_CONVERGED) {  // the increments since the last reliable update
        k_accum_c<<<L.vg, L.vb, 0, s>>>(n, Rpad, active, x.x.p, x.y32.p, nactive);
        ERTGB_CUDA(cudaGetLastError());
    }
    int32_t h_stalled = 0;
    ERTGB_CUDA(cudaMemcpyAsync(&h_stalled, nstalled, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    if (h_stalled) {
        k_zero_restart_c<<<L.vg, L.vb, 0, s>>>(n, Rpad, stalled, x.x.p);
        ERTGB_CUDA(cudaGetLastError());
    }
    return h_stalled;
}

}  // namespace

int complex_response(Context &c, const double *rho_re, const double *rho_im, double *out_re, double *out_im,
                     cudaStream_t s) {
    MeshData &m = c.mesh;
    ComplexState &x = c.cx;
    if (m.n_ext > 0 || !m.ext_rows.empty())
        throw Error(ERTGB_BAD_INPUT, "complex resistivity takes no matrix extension (the reference's complete "
                                     "electrode model is real-valued only, dcfemmodelling.cpp:423-428)");
    for (int32_t cell : c.ent_cell)
        if (cell >= 0) throw Error(ERTGB_BAD_INPUT, "complex resistivity needs node electrodes");
    if (c.ref_elec >= 0 || c.ref_node >= 0 || c.have_fixed)
        throw Error(ERTGB_BAD_INPUT, "complex resistivity with a reference electrode, calibration nodes or "
                                     "Dirichlet boundaries is not supported");
    const int64_t n = m.n, nnz = m.nnz, Rpad = c.Rpad, R = c.R;
    x.have_pot = false;
    // 1 / rho* per cell
    x.sigma.alloc((size_t)m.C);
    DBuf<int32_t> bad;
    bad.alloc(1);
    bad.zero(s);
    k_sigma<<<grid1c(m.C), 256, 0, s>>>(m.C, rho_re, rho_im, x.sigma.p, bad.p);
    ERTGB_CUDA(cudaGetLastError());
    int32_t h_bad = 0;
    ERTGB_CUDA(cudaMemcpyAsync(&h_bad, bad.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    if (h_bad)
        throw Error(ERTGB_BAD_INPUT, "complex response for abs model with negative or zero resistivity is not defined (" +
                                         std::to_string(h_bad) + " cells)");
    // matrices and Jacobi diagonal of every wavenumber
    x.S.alloc((size_t)c.nK * nnz);
    x.dinv.alloc((size_t)c.nK * n);
    k_assemble_c<<<dim3(grid1c(nnz), (unsigned)c.nK), 256, 0, s>>>(
        nnz, m.d_cptr.p, m.d_centry.p, m.d_K.p, m.d_M.p, m.d_bnd_mass.p, c.d_alpha.p, m.d_bnd_cell.p, x.sigma.p,
        c.d_k.p, m.nv * m.nv, m.nvb * m.nvb, m.C, m.B, x.S.p);
    ERTGB_CUDA(cudaGetLastError());
    k_dinv_c<<<grid1c(n * c.nK), 256, 0, s>>>(n, c.nK, nnz, m.d_diag.p, x.S.p, x.dinv.p);
    ERTGB_CUDA(cudaGetLastError());
    CxLaunch L;
    L.n = n;
    L.nnz = nnz;
    L.R = R;
    L.Rpad = Rpad;
    L.NB = (int)std::min<int64_t>(ceil_div(n, kRowsC), kPartC);
    L.vb = dim3(32, kRowsC);
    L.vg = dim3((unsigned)(Rpad / 32), (unsigned)L.NB);
    L.fb = dim3(32, 32);
    L.fg = dim3((unsigned)(Rpad / 32));
    for (DBuf<double2> *v : {&x.x, &x.r, &x.z, &x.p, &x.q}) v->alloc((size_t)n * Rpad);
    x.part.alloc((size_t)5 * L.NB * Rpad);
    x.col.alloc((size_t)C_NCOL * Rpad);
    x.active.alloc((size_t)2 * Rpad + 1);
    x.stalled.alloc((size_t)Rpad + 1);
    ERTGB_CUDA(cudaMemsetAsync(x.col.p, 0, sizeof(double) * C_NCOL * Rpad, s));
    int status = ERTGB_OK;
    x.stalled_columns = 0;
    if (c.precision == ERTGB_PRECISION_MIXED) {
        x.stalled_columns = cocg_mixed(c, L, s, &status);
        if (status == ERTGB_OK && x.stalled_columns > 0) status = cocg_fp64(c, L, s, x.stalled.p);
    } else {
        status = cocg_fp64(c, L, s, nullptr);
    }
    // iterations and the final relative residuals
    int32_t *iters = x.active.p + Rpad;
    std::vector<int32_t> it_h((size_t)Rpad);
    std::vector<double> rr((size_t)Rpad), bb((size_t)Rpad);
    ERTGB_CUDA(cudaMemcpyAsync(it_h.data(), iters, sizeof(int32_t) * Rpad, cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaMemcpyAsync(rr.data(), x.col.p + C_RR * Rpad, sizeof(double) * Rpad, cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaMemcpyAsync(bb.data(), x.col.p + C_BB * Rpad, sizeof(double) * Rpad, cudaMemcpyDeviceToHost, s));
    ERTGB_CUDA(cudaStreamSynchronize(s));
    int maxit = 0;
    double maxres = 0.0;
    for (int64_t t = 0; t < R; t++) {
        maxit = std::max(maxit, it_h[t]);
        if (bb[t] > 0.0) {
            const double rel = std::sqrt(rr[t] / bb[t]);
            if (!std::isfinite(rel)) status = ERTGB_NOT_CONVERGED;
            maxres = std::max(maxres, rel);
        }
    }
    if (maxres > c.rtol * 1.0000001) status = ERTGB_NOT_CONVERGED;
    x.iterations = maxit;
    c.stats.iterations = maxit;
    c.stats.n_rhs = (int32_t)R;
    c.stats.max_rel_residual = maxres;
    c.stats.stalled_columns = x.stalled_columns;
    // collect and response
    x.U.alloc((size_t)c.nE * c.nE);
    k_collect_c<<<(unsigned)ceil_div((int64_t)c.nE * c.nE, 256), 256, 0, s>>>(c.nE, c.nK, Rpad, c.d_enode.p,
                                                                             c.d_w.p, x.x.p, x.U.p);
    k_response_c<<<(unsigned)ceil_div(c.D, 256), 256, 0, s>>>(c.D, c.nE, c.d_abmn.p, c.d_kfac.p, x.U.p, out_re,
                                                              out_im);
    ERTGB_CUDA(cudaGetLastError());
    ERTGB_CUDA(cudaStreamSynchronize(s));
    x.have_pot = true;
    return status;
}

void complex_jacobian(Context &c, const double *m_re, const double *m_im, int n_model, double *J, cudaStream_t s) {
    MeshData &m = c.mesh;
    ComplexState &x = c.cx;
    if (!x.have_pot) throw Error(ERTGB_STATE, "complex jacobian needs a complex response first");
    ERTGB_REQUIRE(m.nv <= 10, "cell node count above 10");
    const bool scale = n_model == (int)m.P;
    ERTGB_REQUIRE(!scale || (m_re && m_im), "null model");
    const unsigned th = 128;
    const dim3 g((unsigned)m.P, (unsigned)ceil_div(c.D, th));
    k_jacobian_c<<<g, th, 0, s>>>(c.D, m.P, c.nE, c.nK, c.Rpad, m.nv, c.d_abmn.p, c.d_kfac.p, m.d_pcell_ptr.p,
                                  m.d_pcell.p, m.d_cells.p, m.d_K.p, m.d_M.p, c.d_k.p, c.d_w.p, x.x.p,
                                  scale ? m_re : nullptr, scale ? m_im : nullptr, reinterpret_cast<double2 *>(J));
    ERTGB_CUDA(cudaGetLastError());
    ERTGB_CUDA(cudaStreamSynchronize(s));
}

}  // namespace ertgb
