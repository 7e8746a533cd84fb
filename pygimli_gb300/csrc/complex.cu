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

namespace ertgb {
namespace {

constexpr double kTolC = 1e-12;  // TOLERANCE of the reference (gimli.h)
constexpr int kRowsC = 8;        // rows per block in the vector kernels
constexpr int kPartC = 608;      // block partial rows of the column reductions
constexpr int kGraphItersC = 16; // iterations per CUDA graph launch

// per-column scalars (x Rpad)
enum CCol { C_RHO_RE = 0, C_RHO_IM, C_ALPHA_RE, C_ALPHA_IM, C_BETA_RE, C_BETA_IM, C_BB, C_RR, C_NCOL };

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

// z = D^-1 r; with SETP also p = z.  Partials of r^T z (complex) and r^H r.
template <bool SETP>
__global__ void k_precond_c(int64_t n, int nE, int64_t R, int64_t Rpad, const double2 *__restrict__ dinv,
                            const int32_t *__restrict__ active, const double2 *__restrict__ r,
                            double2 *__restrict__ z, double2 *__restrict__ p, double *__restrict__ p_re,
                            double *__restrict__ p_im, double *__restrict__ p_rr) {
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const bool act = t < R && (SETP || active[t]);
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
__global__ void k_finish_init_c(int64_t Rpad, int64_t R, int NB, const double *__restrict__ p_re,
                                const double *__restrict__ p_im, const double *__restrict__ p_rr,
                                double *__restrict__ col, int32_t *__restrict__ active, int32_t *__restrict__ iters,
                                int32_t *__restrict__ nactive) {
    __shared__ double ra[32][33], rb[32][33], rc[32][33];
    const int64_t t = (int64_t)blockIdx.x * 32 + threadIdx.x;
    const double re = col_sum(p_re, NB, Rpad, t, ra);
    const double im = col_sum(p_im, NB, Rpad, t, rb);
    const double rr = col_sum(p_rr, NB, Rpad, t, rc);
    if (threadIdx.y != 0) return;
    col[C_RHO_RE * Rpad + t] = re;
    col[C_RHO_IM * Rpad + t] = im;
    col[C_BB * Rpad + t] = rr;
    col[C_RR * Rpad + t] = rr;
    const int a = (t < R && rr > 0.0) ? 1 : 0;
    active[t] = a;
    iters[t] = 0;
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

int complex_response(Context &c, const double *rho_re, const double *rho_im, double *out_re, double *out_im,
                     cudaStream_t s) {
    MeshData &m = c.mesh;
    ComplexState &x = c.cx;
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
    // block COCG
    const int NB = (int)std::min<int64_t>(ceil_div(n, kRowsC), kPartC);
    for (DBuf<double2> *v : {&x.x, &x.r, &x.z, &x.p, &x.q}) v->alloc((size_t)n * Rpad);
    x.part.alloc((size_t)5 * NB * Rpad);
    x.col.alloc((size_t)C_NCOL * Rpad);
    x.active.alloc((size_t)2 * Rpad + 1);
    double *pa = x.part.p, *pb = pa + (size_t)NB * Rpad, *pc = pb + (size_t)NB * Rpad;
    double *pd = pc + (size_t)NB * Rpad, *pe = pd + (size_t)NB * Rpad;
    int32_t *active = x.active.p, *iters = active + Rpad, *nactive = active + 2 * Rpad;
    ERTGB_CUDA(cudaMemsetAsync(x.x.p, 0, sizeof(double2) * n * Rpad, s));
    ERTGB_CUDA(cudaMemsetAsync(x.r.p, 0, sizeof(double2) * n * Rpad, s));
    ERTGB_CUDA(cudaMemsetAsync(x.col.p, 0, sizeof(double) * C_NCOL * Rpad, s));
    ERTGB_CUDA(cudaMemsetAsync(nactive, 0, sizeof(int32_t), s));
    k_sources_c<<<(unsigned)ceil_div(R, 256), 256, 0, s>>>(c.nE, R, Rpad, c.d_enode.p, x.r.p);
    const dim3 vb(32, kRowsC), vg((unsigned)(Rpad / 32), (unsigned)NB), fb(32, 32), fg((unsigned)(Rpad / 32));
    k_precond_c<true><<<vg, vb, 0, s>>>(n, c.nE, R, Rpad, x.dinv.p, active, x.r.p, x.z.p, x.p.p, pa, pb, pc);
    k_finish_init_c<<<fg, fb, 0, s>>>(Rpad, R, NB, pa, pb, pc, x.col.p, active, iters, nactive);
    ERTGB_CUDA(cudaGetLastError());
    const double rtol2 = c.rtol * c.rtol;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    int status = ERTGB_OK;
    try {
        ERTGB_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int it = 0; it < kGraphItersC; it++) {
            k_spmm_c<<<vg, vb, 0, s>>>(n, nnz, c.nE, R, Rpad, m.d_rowptr.p, m.d_colidx.p, x.S.p, active, x.p.p, x.q.p,
                                       pd, pe);
            k_finish_alpha_c<<<fg, fb, 0, s>>>(Rpad, NB, pd, pe, x.col.p, active, nactive);
            k_update_xr_c<<<vg, vb, 0, s>>>(n, Rpad, x.col.p, active, x.x.p, x.r.p, x.p.p, x.q.p);
            k_precond_c<false><<<vg, vb, 0, s>>>(n, c.nE, R, Rpad, x.dinv.p, active, x.r.p, x.z.p, nullptr, pa, pb,
                                                 pc);
            k_finish_beta_c<<<fg, fb, 0, s>>>(Rpad, NB, rtol2, pa, pb, pc, x.col.p, active, iters, nactive);
            k_update_p_c<<<vg, vb, 0, s>>>(n, Rpad, x.col.p, active, x.z.p, x.p.p);
        }
        ERTGB_CUDA(cudaStreamEndCapture(s, &g));
        ERTGB_CUDA(cudaGraphInstantiate(&ge, g, 0));
        int32_t h_active = 0;
        ERTGB_CUDA(cudaMemcpyAsync(&h_active, nactive, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
        ERTGB_CUDA(cudaStreamSynchronize(s));
        int done = 0;
        while (h_active > 0) {
            if (done >= c.max_iter) {
                status = ERTGB_NOT_CONVERGED;
                break;
            }
            for (int u = 0; u < 4; u++) ERTGB_CUDA(cudaGraphLaunch(ge, s));
            done += 4 * kGraphItersC;
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
    // iterations and the final relative residuals
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
