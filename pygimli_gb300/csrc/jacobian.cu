// Reciprocity Jacobian of the DC forward operator (FP64).
//
//   J[d, p] = sum_{cells c with marker p} sum_k w_k
//             ((K_c + k^2 M_c)(u_a,k - u_b,k)) . (u_m,k - u_n,k)
//   then J[d, p] /= (model_p^2 / kfac_d) when the model has one value per
//   parameter.
// Reference: createSensitivityCol_ / CreateSensitivityColMT::calc2
// (core/src/bert/bertJacobian.cpp:70-119, 267-421), ElementMatrix::mult
// (core/src/elementmatrix.h:280-293), scaling in
// core/src/bert/dcfemmodelling.cpp:1377-1384.  Potentials are the
// sub-potentials of the last response (column k*nE + e of the n x Rpad
// block); an electrode index -1 contributes a zero potential.
//
// Layout: one block per tile of consecutive parameters (at most 32, their
// cells within the shared-memory budget).  The block stages, for each cell of
// the tile and each wavenumber, the node potentials U[i][e] of every
// electrode (plus a zero column for index -1) and V = S U, then threads walk
// the (datum, parameter) pairs with the parameter fastest, so that each warp
// writes contiguous runs of a J row.
#include <algorithm>

#include "ertgb_internal.cuh"

namespace ertgb {

namespace {

template <int NV, typename OutT>
__global__ void __launch_bounds__(256)
    k_jacobian(const int32_t *__restrict__ tile_p, const int32_t *__restrict__ pcell_ptr,
               const int32_t *__restrict__ pcell, const int32_t *__restrict__ cells,
               const double *__restrict__ K, const double *__restrict__ M, const double *__restrict__ kv,
               const double *__restrict__ w, int nK, int nE, int64_t Rpad, const double *__restrict__ pot,
               const int32_t *__restrict__ abmn, const double *__restrict__ kfac,
               const double *__restrict__ model, int64_t P, int64_t D, int max_cells, OutT *__restrict__ J) {
    extern __shared__ double smem[];
    const int E1 = nE + 1;
    const int per_cell = nK * NV * E1;  // doubles per cell for U (same for V)
    double *U = smem;
    double *V = smem + (size_t)max_cells * per_cell;
    const int64_t p0 = tile_p[blockIdx.x], p1 = tile_p[blockIdx.x + 1];
    const int TP = (int)(p1 - p0);
    const int cbeg = pcell_ptr[p0], cend = pcell_ptr[p1];
    const int ncell = cend - cbeg;
    const int nchunks = (ncell + max_cells - 1) / max_cells;
    const int64_t pairs = D * TP;
    const int64_t nbatch = (pairs + blockDim.x - 1) / blockDim.x;

    auto stage = [&](int c0, int cn) {
        // potentials at the cell nodes
        const int total = cn * per_cell;
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int lc = idx / per_cell;
            int rem = idx - lc * per_cell;
            const int ki = rem / (NV * E1);
            rem -= ki * NV * E1;
            const int i = rem / E1;
            const int e = rem - i * E1;
            const int cell = pcell[cbeg + c0 + lc];
            const int64_t node = cells[(int64_t)cell * NV + i];
            U[idx] = (e < nE) ? pot[node * Rpad + (int64_t)ki * nE + e] : 0.0;
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int lc = idx / per_cell;
            int rem = idx - lc * per_cell;
            const int ki = rem / (NV * E1);
            rem -= ki * NV * E1;
            const int i = rem / E1;
            const int e = rem - i * E1;
            const int cell = pcell[cbeg + c0 + lc];
            const double k = kv[ki];
            const double kk = k * k;
            const double *Kc = K + (int64_t)cell * NV * NV + i * NV;
            const double *Mc = M + (int64_t)cell * NV * NV + i * NV;
            const double *Uc = U + (size_t)lc * per_cell + (size_t)ki * NV * E1 + e;
            double acc = 0.0;
#pragma unroll
            for (int j = 0; j < NV; j++) acc = fma(Mc[j] * kk + Kc[j], Uc[j * E1], acc);
            V[idx] = acc;
        }
        __syncthreads();
    };

    auto accumulate = [&](int64_t pr, int c0, int cn, double acc) -> double {
        const int pl = (int)(pr % TP);
        const int64_t d = pr / TP;
        const int64_t p = p0 + pl;
        int a = abmn[4 * d], b = abmn[4 * d + 1], m = abmn[4 * d + 2], n = abmn[4 * d + 3];
        a = a < 0 ? nE : a;
        b = b < 0 ? nE : b;
        m = m < 0 ? nE : m;
        n = n < 0 ? nE : n;
        const int lo = max(pcell_ptr[p] - cbeg, c0), hi = min(pcell_ptr[p + 1] - cbeg, c0 + cn);
        for (int lc = lo; lc < hi; lc++) {
            const double *Ub = U + (size_t)(lc - c0) * per_cell;
            const double *Vb = V + (size_t)(lc - c0) * per_cell;
            for (int ki = 0; ki < nK; ki++) {
                const double *Uk = Ub + (size_t)ki * NV * E1;
                const double *Vk = Vb + (size_t)ki * NV * E1;
                double s = 0.0;
#pragma unroll
                for (int i = 0; i < NV; i++)
                    s = fma(Vk[i * E1 + a] - Vk[i * E1 + b], Uk[i * E1 + m] - Uk[i * E1 + n], s);
                acc = fma(s, w[ki], acc);
            }
        }
        return acc;
    };

    auto store = [&](int64_t pr, double acc) {
        const int pl = (int)(pr % TP);
        const int64_t d = pr / TP;
        const int64_t p = p0 + pl;
        if (model) {
            const double m = model[p];
            acc = acc / ((m * m) / kfac[d]);
        }
        J[d * P + p] = (OutT)acc;
    };

    if (nchunks <= 1) {
        if (ncell > 0) stage(0, ncell);
        for (int64_t pr = threadIdx.x; pr < pairs; pr += blockDim.x) store(pr, accumulate(pr, 0, ncell, 0.0));
    } else {
        for (int64_t bt = 0; bt < nbatch; bt++) {
            const int64_t pr = bt * blockDim.x + threadIdx.x;
            double acc = 0.0;
            for (int ch = 0; ch < nchunks; ch++) {
                const int c0 = ch * max_cells;
                const int cn = min(max_cells, ncell - c0);
                __syncthreads();
                stage(c0, cn);
                if (pr < pairs) acc = accumulate(pr, c0, cn, acc);
            }
            if (pr < pairs) store(pr, acc);
        }
    }
}

template <typename OutT>
void launch(Context &c, const double *model, OutT *J, cudaStream_t s) {
    MeshData &m = c.mesh;
    const int ntiles = (int)m.jtile_p.size() - 1;
    if (ntiles <= 0) return;
    const size_t per_cell = (size_t)c.nK * m.nv * (c.nE + 1);
    const size_t smem = 2 * per_cell * m.jtile_cells_max * sizeof(double);
    if (smem > 227 * 1024)
        throw Error(ERTGB_BAD_INPUT, "Jacobian staging of one cell exceeds shared memory (too many electrodes x wavenumbers)");
    if (m.nv == 3) {
        auto kern = k_jacobian<3, OutT>;
        ERTGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<ntiles, 256, smem, s>>>(m.d_jtile_p.p, m.d_pcell_ptr.p, m.d_pcell.p, m.d_cells.p, m.d_K.p, m.d_M.p,
                                       c.d_k.p, c.d_w.p, c.nK, c.nE, c.Rpad, c.d_x.p, c.d_abmn.p, c.d_kfac.p, model,
                                       m.P, c.D, m.jtile_cells_max, J);
    } else {
        auto kern = k_jacobian<4, OutT>;
        ERTGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<ntiles, 256, smem, s>>>(m.d_jtile_p.p, m.d_pcell_ptr.p, m.d_pcell.p, m.d_cells.p, m.d_K.p, m.d_M.p,
                                       c.d_k.p, c.d_w.p, c.nK, c.nE, c.Rpad, c.d_x.p, c.d_abmn.p, c.d_kfac.p, model,
                                       m.P, c.D, m.jtile_cells_max, J);
    }
    ERTGB_CUDA(cudaGetLastError());
}

}  // namespace

void jacobian(Context &c, const double *model, int n_model, void *J, int dtype, cudaStream_t s) {
    const double *mdl = (n_model == c.mesh.P) ? model : nullptr;
    if (dtype == 0) launch<double>(c, mdl, (double *)J, s);
    else launch<float>(c, mdl, (float *)J, s);
}

void profile_jacobian(Context &c, int reps, double *J, double *ms, double *bytes, double *flops) {
    if (!c.have_pot) throw Error(ERTGB_STATE, "profile needs a completed response");
    MeshData &m = c.mesh;
    cudaStream_t s = c.stream;
    launch<double>(c, nullptr, J, s);
    ERTGB_CUDA(cudaEventRecord(c.ev[0], s));
    for (int r = 0; r < reps; r++) launch<double>(c, nullptr, J, s);
    ERTGB_CUDA(cudaEventRecord(c.ev[1], s));
    ERTGB_CUDA(cudaEventSynchronize(c.ev[1]));
    float t = 0.f;
    ERTGB_CUDA(cudaEventElapsedTime(&t, c.ev[0], c.ev[1]));
    *ms = (double)t / reps;
    const double Ca = (double)m.pcell.size();
    // J written once, potentials read once, cell nodes + element matrices,
    // parameter->cell map, scheme
    *bytes = (double)c.D * m.P * 8.0 + (double)m.n * c.Rpad * 8.0 + Ca * (m.nv * 4.0 + 2.0 * m.nv * m.nv * 8.0 + 4.0) +
             (double)(m.P + 1) * 4.0 + (double)c.D * (16.0 + 8.0);
    // V = S U per (cell, k, electrode) and the (datum, cell, k) products
    *flops = Ca * c.nK * (c.nE + 1) * m.nv * (2.0 * m.nv + 2.0) + (double)c.D * Ca * c.nK * (m.nv * 4.0 + 2.0);
}

}  // namespace ertgb
