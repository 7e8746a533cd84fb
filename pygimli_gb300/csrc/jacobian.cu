// Reciprocity Jacobian of the DC forward operator.
//
//   J[d, p] = sum_{cells c with marker p} sum_k w_k
//             ((K_c + k^2 M_c)(u_a,k - u_b,k)) . (u_m,k - u_n,k)
//   then J[d, p] *= kfac_d / model_p^2 when the model has one value per
//   parameter (the reference divides by model_p^2 / kfac_d).
// Reference: createSensitivityCol_ / CreateSensitivityColMT::calc2
// (core/src/bert/bertJacobian.cpp:70-119, 267-421), ElementMatrix::mult
// (core/src/elementmatrix.h:280-293), scaling in
// core/src/bert/dcfemmodelling.cpp:1377-1384.  Potentials are the
// sub-potentials of the last response (column k*nE + e of the n x Rpad
// block); an electrode index -1 contributes a zero potential.
//
// Dipole tables: a scheme uses far fewer distinct current dipoles (a, b) and
// potential dipoles (m, n) than data.  One block handles a tile of
// consecutive parameters.  For each cell of the tile and each wavenumber it
// stages the node potentials U[i][e] of every electrode, V = S U, and then
// the FP64 differences
//   TA[ia][i] = V[a][i] - V[b][i]   for every distinct current dipole,
//   TM[im][i] = U[m][i] - U[n][i]   for every distinct potential dipole,
// stored with the cell index fastest (conflict-free shared-memory reads).
// Every (datum, parameter) pair is then an nv-term dot product of two table
// rows.  The differences are formed in FP64 (they cancel); the FP32 form
// rounds the differences to FP32 and accumulates and stores in FP32.
// Threads walk (datum, parameter) pairs with the parameter fastest, so a
// warp writes contiguous runs of a J row.
#include <algorithm>

#include "ertgb_internal.cuh"

namespace ertgb {

namespace {

template <int NV, typename CT>
__global__ void __launch_bounds__(256)
    k_jacobian(const int32_t *__restrict__ tile_p, const int32_t *__restrict__ pcell_ptr,
               const int32_t *__restrict__ pcell, const int32_t *__restrict__ cells,
               const double *__restrict__ K, const double *__restrict__ M, const double *__restrict__ kv,
               const double *__restrict__ w, int nK, int nE, int64_t Rpad, const double *__restrict__ pot,
               int nA, const int32_t *__restrict__ dip_a, int nM, const int32_t *__restrict__ dip_m,
               const int32_t *__restrict__ data_dip, const CT *__restrict__ scale_d,
               const CT *__restrict__ scale_p, int64_t P, int64_t D, int max_cells, CT *__restrict__ J) {
    extern __shared__ double smem[];
    const int E1 = nE + 1;
    const int uv_cell = nK * NV * E1;  // doubles per cell for U (same for V)
    double *U = smem;
    double *V = smem + (size_t)max_cells * uv_cell;
    CT *TA = reinterpret_cast<CT *>(V + (size_t)max_cells * uv_cell);
    CT *TM = TA + (size_t)nK * nA * NV * max_cells;
    const int64_t p0 = tile_p[blockIdx.x], p1 = tile_p[blockIdx.x + 1];
    const int TP = (int)(p1 - p0);
    const int cbeg = pcell_ptr[p0], cend = pcell_ptr[p1];
    const int ncell = cend - cbeg;
    const int nchunks = (ncell + max_cells - 1) / max_cells;
    const int64_t pairs = D * TP;
    const int64_t nbatch = (pairs + blockDim.x - 1) / blockDim.x;
    const int W = max_cells;  // row stride of the tables (cell fastest)

    auto stage = [&](int c0, int cn) {
        const int total = cn * uv_cell;
        for (int idx = threadIdx.x; idx < total; idx += blockDim.x) {
            const int lc = idx / uv_cell;
            int rem = idx - lc * uv_cell;
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
            const int lc = idx / uv_cell;
            int rem = idx - lc * uv_cell;
            const int ki = rem / (NV * E1);
            rem -= ki * NV * E1;
            const int i = rem / E1;
            const int e = rem - i * E1;
            const int cell = pcell[cbeg + c0 + lc];
            const double k = kv[ki];
            const double kk = k * k;
            const double *Kc = K + (int64_t)cell * NV * NV + i * NV;
            const double *Mc = M + (int64_t)cell * NV * NV + i * NV;
            const double *Uc = U + (size_t)lc * uv_cell + (size_t)ki * NV * E1 + e;
            double acc = 0.0;
#pragma unroll
            for (int j = 0; j < NV; j++) acc = fma(Mc[j] * kk + Kc[j], Uc[j * E1], acc);
            V[idx] = acc;
        }
        __syncthreads();
        // dipole tables, FP64 differences
        const int ta = nK * nA * NV * cn;
        for (int idx = threadIdx.x; idx < ta; idx += blockDim.x) {
            const int lc = idx % cn;
            int rem = idx / cn;
            const int i = rem % NV;
            rem /= NV;
            const int ia = rem % nA;
            const int ki = rem / nA;
            int a = dip_a[2 * ia], b = dip_a[2 * ia + 1];
            a = a < 0 ? nE : a;
            b = b < 0 ? nE : b;
            const double *Vc = V + (size_t)lc * uv_cell + ((size_t)ki * NV + i) * E1;
            TA[(((size_t)ki * nA + ia) * NV + i) * W + lc] = (CT)(Vc[a] - Vc[b]);
        }
        const int tm = nK * nM * NV * cn;
        for (int idx = threadIdx.x; idx < tm; idx += blockDim.x) {
            const int lc = idx % cn;
            int rem = idx / cn;
            const int i = rem % NV;
            rem /= NV;
            const int im = rem % nM;
            const int ki = rem / nM;
            int m = dip_m[2 * im], n = dip_m[2 * im + 1];
            m = m < 0 ? nE : m;
            n = n < 0 ? nE : n;
            const double *Uc = U + (size_t)lc * uv_cell + ((size_t)ki * NV + i) * E1;
            TM[(((size_t)ki * nM + im) * NV + i) * W + lc] = (CT)(Uc[m] - Uc[n]);
        }
        __syncthreads();
    };

    auto accumulate = [&](int64_t pr, int c0, int cn, CT acc) -> CT {
        const int pl = (int)(pr % TP);
        const int64_t d = pr / TP;
        const int64_t p = p0 + pl;
        const int ia = data_dip[2 * d], im = data_dip[2 * d + 1];
        const int lo = max(pcell_ptr[p] - cbeg, c0), hi = min(pcell_ptr[p + 1] - cbeg, c0 + cn);
        for (int lc = lo - c0; lc < hi - c0; lc++) {
            for (int ki = 0; ki < nK; ki++) {
                const CT *ta = TA + ((size_t)ki * nA + ia) * NV * W + lc;
                const CT *tm = TM + ((size_t)ki * nM + im) * NV * W + lc;
                CT s = 0;
#pragma unroll
                for (int i = 0; i < NV; i++) s = fma(ta[i * W], tm[i * W], s);
                acc = fma(s, (CT)w[ki], acc);
            }
        }
        return acc;
    };

    auto store = [&](int64_t pr, CT acc) {
        const int pl = (int)(pr % TP);
        const int64_t d = pr / TP;
        const int64_t p = p0 + pl;
        if (scale_p) acc = (acc * scale_d[d]) * scale_p[p];
        J[d * P + p] = acc;
    };

    if (nchunks <= 1) {
        if (ncell > 0) stage(0, ncell);
        for (int64_t pr = threadIdx.x; pr < pairs; pr += blockDim.x) store(pr, accumulate(pr, 0, ncell, (CT)0));
    } else {
        for (int64_t bt = 0; bt < nbatch; bt++) {
            const int64_t pr = bt * blockDim.x + threadIdx.x;
            CT acc = 0;
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

// scale_d[d] = kfac[d], scale_p[p] = 1 / model[p]^2 in the compute type
template <typename CT>
__global__ void k_jac_scales(int64_t D, int64_t P, const double *__restrict__ kfac,
                             const double *__restrict__ model, CT *__restrict__ sd, CT *__restrict__ sp) {
    const int64_t total = D + P;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        if (t < D) {
            sd[t] = (CT)kfac[t];
        } else {
            const double m = model[t - D];
            sp[t - D] = (CT)(1.0 / (m * m));
        }
    }
}

size_t jac_cell_bytes(const Context &c, int dtype) {
    const size_t uv = 2 * (size_t)c.nK * c.mesh.nv * (c.nE + 1) * sizeof(double);
    const size_t tab = (size_t)c.nK * (c.nA + c.nM) * c.mesh.nv * (dtype == 0 ? 8 : 4);
    return uv + tab;
}

template <typename CT>
void launch(Context &c, const double *model, CT *J, int dtype, cudaStream_t s) {
    MeshData &m = c.mesh;
    JacTiles &T = c.jtiles[dtype];
    const int ntiles = (int)T.tile_p.size() - 1;
    if (ntiles <= 0) return;
    const size_t smem = jac_cell_bytes(c, dtype) * T.max_cells;
    const CT *sd = nullptr, *sp = nullptr;
    if (model) {
        c.d_jscale.alloc((size_t)(c.D + m.P) * sizeof(CT));
        CT *base = reinterpret_cast<CT *>(c.d_jscale.p);
        k_jac_scales<CT><<<(unsigned)std::min<int64_t>(ceil_div(c.D + m.P, 256), 4096), 256, 0, s>>>(
            c.D, m.P, c.d_kfac.p, model, base, base + c.D);
        ERTGB_CUDA(cudaGetLastError());
        sd = base;
        sp = base + c.D;
    }
    auto go = [&](auto kern) {
        ERTGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        kern<<<ntiles, 256, smem, s>>>(T.d_tile_p.p, m.d_pcell_ptr.p, m.d_pcell.p, m.d_cells.p, m.d_K.p, m.d_M.p,
                                       c.d_k.p, c.d_w.p, c.nK, c.nE, c.Rpad, c.d_x.p, c.nA, c.d_dip_a.p, c.nM,
                                       c.d_dip_m.p, c.d_data_dip.p, sd, sp, m.P, c.D, T.max_cells, J);
        ERTGB_CUDA(cudaGetLastError());
    };
    if (m.nv == 3) go(k_jacobian<3, CT>);
    else go(k_jacobian<4, CT>);
}

}  // namespace

// Parameter -> cells and the Jacobian tiles of both table precisions
// (consecutive parameters whose cells fit the shared-memory budget).
void build_jacobian_tiles(Context &c) {
    MeshData &m = c.mesh;
    const int64_t P = m.P;
    m.pcell_ptr.assign(P + 1, 0);
    for (int64_t i = 0; i < m.C; i++)
        if (m.marker[i] >= 0) m.pcell_ptr[m.marker[i] + 1]++;
    for (int64_t p = 0; p < P; p++) m.pcell_ptr[p + 1] += m.pcell_ptr[p];
    m.pcell.assign(m.pcell_ptr[P], 0);
    std::vector<int32_t> pos(m.pcell_ptr.begin(), m.pcell_ptr.end() - 1);
    for (int64_t i = 0; i < m.C; i++)
        if (m.marker[i] >= 0) m.pcell[pos[m.marker[i]]++] = (int32_t)i;
    m.d_pcell_ptr.upload(m.pcell_ptr, c.stream);
    m.d_pcell.upload(m.pcell, c.stream);
    const size_t budget = 200 * 1024;
    for (int dt = 0; dt < 2; dt++) {
        JacTiles &T = c.jtiles[dt];
        const size_t per_cell = jac_cell_bytes(c, dt);
        T.max_cells = per_cell > budget ? 0 : (int)std::min<size_t>(32, budget / per_cell);
        T.tile_p.assign(1, 0);
        if (T.max_cells == 0) continue;
        int64_t p = 0;
        while (p < P) {
            int64_t q = p, ncell = 0;
            while (q < P && q - p < 32) {
                const int64_t cq = m.pcell_ptr[q + 1] - m.pcell_ptr[q];
                if (q > p && ncell + cq > T.max_cells) break;
                ncell += cq;
                q++;
            }
            if (q == p) q = p + 1;
            T.tile_p.push_back((int32_t)q);
            p = q;
        }
        T.d_tile_p.upload(T.tile_p, c.stream);
    }
}

void jacobian(Context &c, const double *model, int n_model, void *J, int dtype, cudaStream_t s) {
    if (c.jtiles[dtype].max_cells == 0)
        throw Error(ERTGB_BAD_INPUT, "Jacobian staging of one cell exceeds shared memory "
                                     "(too many electrodes x wavenumbers x dipoles)");
    const double *mdl = (n_model == c.mesh.P) ? model : nullptr;
    if (dtype == 0) launch<double>(c, mdl, (double *)J, 0, s);
    else launch<float>(c, mdl, (float *)J, 1, s);
}

void profile_jacobian(Context &c, int reps, double *J, double *ms, double *bytes, double *flops) {
    if (!c.have_pot) throw Error(ERTGB_STATE, "profile needs a completed response");
    MeshData &m = c.mesh;
    cudaStream_t s = c.stream;
    launch<double>(c, nullptr, J, 0, s);
    ERTGB_CUDA(cudaEventRecord(c.ev[0], s));
    for (int r = 0; r < reps; r++) launch<double>(c, nullptr, J, 0, s);
    ERTGB_CUDA(cudaEventRecord(c.ev[1], s));
    ERTGB_CUDA(cudaEventSynchronize(c.ev[1]));
    float t = 0.f;
    ERTGB_CUDA(cudaEventElapsedTime(&t, c.ev[0], c.ev[1]));
    *ms = (double)t / reps;
    const double Ca = (double)m.pcell.size();
    // J written once, potentials read once, cell nodes + element matrices,
    // parameter->cell map, scheme and its dipole indices
    *bytes = (double)c.D * m.P * 8.0 + (double)m.n * c.Rpad * 8.0 + Ca * (m.nv * 4.0 + 2.0 * m.nv * m.nv * 8.0 + 4.0) +
             (double)(m.P + 1) * 4.0 + (double)c.D * (8.0 + 8.0) + (double)(c.nA + c.nM) * 8.0;
    // V = S U, the dipole differences, and one nv-term dot per (datum, cell, k)
    *flops = Ca * c.nK * ((c.nE + 1) * m.nv * 2.0 * m.nv + (c.nA + c.nM) * m.nv) +
             (double)c.D * Ca * c.nK * (m.nv * 2.0 + 2.0);
}

}  // namespace ertgb
