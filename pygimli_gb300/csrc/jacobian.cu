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
// potential dipoles (m, n) than data.  One block handles a tile of up to TW
// consecutive parameters (TW cells).  For G cells at a time it stages the
// node potentials U[i][e] of every electrode and V = S U in FP64, then forms
// the FP64 differences
//   TA[ia][i] = V[a][i] - V[b][i]   for every distinct current dipole,
//   TM[im][i] = U[m][i] - U[n][i]   for every distinct potential dipole,
// stored with the cell index fastest.  Every (datum, parameter) pair is then
// an nv-term dot product of two table rows per wavenumber.  The differences
// are formed in FP64 (they cancel); the FP32 form rounds them to FP32 and
// accumulates and stores in FP32.  Lane layout in the pair phase: lane =
// (datum sub-row, cell) with the cell fastest, so conflict-free table reads
// and contiguous runs of a J row per sub-row.
#include <algorithm>
#include <map>
#include <type_traits>

#include "ertgb_internal.cuh"

namespace ertgb {

namespace {

constexpr int kThreads = 512;
constexpr size_t kSmemBudget = 110 * 1024;       // two blocks per SM
constexpr size_t kSmemBudgetLarge = 220 * 1024;  // one block per SM (many wavenumbers x dipoles)

template <int NV, typename CT, int TW>
__global__ void __launch_bounds__(kThreads)
    k_jacobian(const int32_t *__restrict__ tile_p, const int32_t *__restrict__ pcell_ptr,
               const int32_t *__restrict__ pcell, const int32_t *__restrict__ cells,
               const double *__restrict__ K, const double *__restrict__ M, const double *__restrict__ kv,
               const double *__restrict__ w, int nK, int nE, int64_t Rpad, const double *__restrict__ pot,
               int nA, const int32_t *__restrict__ dip_a, int nM, const int32_t *__restrict__ dip_m,
               const int32_t *__restrict__ data_dip, const CT *__restrict__ scale_d,
               const CT *__restrict__ scale_p, int64_t P, int64_t D, int G, CT *__restrict__ J) {
    extern __shared__ double smem[];
    const int E1 = nE + 1;
    const int uv_cell = nK * NV * E1;  // doubles per staged cell (U; V the same)
    double *U = smem;
    double *V = smem + (size_t)G * uv_cell;
    CT *TA = reinterpret_cast<CT *>(V + (size_t)G * uv_cell);
    CT *TM = TA + (size_t)nK * nA * NV * TW;
    const int p0 = tile_p[blockIdx.x], p1 = tile_p[blockIdx.x + 1];
    const int TP = p1 - p0;
    const int cbeg = pcell_ptr[p0];
    const int ncell = pcell_ptr[p1] - cbeg;
    const int nchunks = (ncell + TW - 1) / TW;

    // pair-phase lane layout
    constexpr int SUB = 32 / TW;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = lane % TW, sub = lane / TW;
    const int dstep = (kThreads / 32) * SUB;
    const int d0 = warp * SUB + sub;
    const bool has_p = c < TP;
    const int p = p0 + (has_p ? c : 0);
    const int pc0 = pcell_ptr[p] - cbeg, pc1 = pcell_ptr[p + 1] - cbeg;  // this parameter's cells in the tile
    const CT sp = (scale_p && has_p) ? scale_p[p] : (CT)1;
    __shared__ CT wk[64];  // wavenumber weights (nK <= 64)
    for (int ki = threadIdx.x; ki < nK; ki += kThreads) wk[ki] = (CT)w[ki];
    __syncthreads();

    // stage cells [c0 + g0, c0 + g0 + gn) and write their table columns g0.. of the chunk
    auto build = [&](int c0, int cn) {
        for (int g0 = 0; g0 < cn; g0 += G) {
            const int gn = min(G, cn - g0);
            __syncthreads();
            for (int q = threadIdx.x; q < gn * uv_cell; q += kThreads) {
                const int g = q / uv_cell;
                const int rem = q - g * uv_cell;
                const int kin = rem / E1;  // ki * NV + i
                const int e = rem - kin * E1;
                const int ki = kin / NV, i = kin - ki * NV;
                const int cell = pcell[cbeg + c0 + g0 + g];
                const int64_t node = cells[(int64_t)cell * NV + i];
                U[q] = (e < nE) ? pot[node * Rpad + (int64_t)ki * nE + e] : 0.0;
            }
            __syncthreads();
            for (int q = threadIdx.x; q < gn * uv_cell; q += kThreads) {
                const int g = q / uv_cell;
                const int rem = q - g * uv_cell;
                const int kin = rem / E1;
                const int e = rem - kin * E1;
                const int ki = kin / NV, i = kin - ki * NV;
                const int cell = pcell[cbeg + c0 + g0 + g];
                const double k = kv[ki];
                const double kk = k * k;
                const double *Kc = K + (int64_t)cell * NV * NV + i * NV;
                const double *Mc = M + (int64_t)cell * NV * NV + i * NV;
                const double *Uc = U + (size_t)g * uv_cell + (size_t)ki * NV * E1 + e;
                double acc = 0.0;
#pragma unroll
                for (int j = 0; j < NV; j++) acc = fma(Mc[j] * kk + Kc[j], Uc[j * E1], acc);
                V[q] = acc;
            }
            __syncthreads();
            const int rowsA = nK * nA * NV, rowsM = nK * nM * NV;
            for (int q = threadIdx.x; q < (rowsA + rowsM) * gn; q += kThreads) {
                const int g = q % gn;
                int row = q / gn;
                const bool isA = row < rowsA;
                if (!isA) row -= rowsA;
                const int i = row % NV;
                const int kd = row / NV;  // ki * n{A,M} + dipole
                const int nd = isA ? nA : nM;
                const int ki = kd / nd, dp = kd - ki * nd;
                const int32_t *dip = isA ? dip_a : dip_m;
                int a = dip[2 * dp], b = dip[2 * dp + 1];
                a = a < 0 ? nE : a;
                b = b < 0 ? nE : b;
                const double *src = (isA ? V : U) + (size_t)g * uv_cell + ((size_t)ki * NV + i) * E1;
                CT *dst = isA ? TA : TM;
                dst[(size_t)row * TW + g0 + g] = (CT)(src[a] - src[b]);
            }
        }
        __syncthreads();
    };

    auto pair_sum = [&](int64_t d, int lo, int hi) -> CT {
        const int ia = data_dip[2 * d], im = data_dip[2 * d + 1];
        CT acc = 0;
        for (int lc = lo; lc < hi; lc++) {
            for (int ki = 0; ki < nK; ki++) {
                const CT *ta = TA + ((size_t)ki * nA + ia) * NV * TW + lc;
                const CT *tm = TM + ((size_t)ki * nM + im) * NV * TW + lc;
                CT s = 0;
#pragma unroll
                for (int i = 0; i < NV; i++) s = fma(ta[i * TW], tm[i * TW], s);
                acc = fma(s, wk[ki], acc);
            }
        }
        return acc;
    };

    if (nchunks <= 1) {
        if (ncell > 0) build(0, ncell);
        if (has_p) {
            int64_t d = d0;
            for (; d + dstep < D; d += 2 * dstep) {  // two independent rows in flight
                CT a0 = pair_sum(d, pc0, pc1);
                CT a1 = pair_sum(d + dstep, pc0, pc1);
                if (scale_p) {
                    a0 = (a0 * scale_d[d]) * sp;
                    a1 = (a1 * scale_d[d + dstep]) * sp;
                }
                J[d * P + p] = a0;
                J[(d + dstep) * P + p] = a1;
            }
            if (d < D) {
                CT a0 = pair_sum(d, pc0, pc1);
                if (scale_p) a0 = (a0 * scale_d[d]) * sp;
                J[d * P + p] = a0;
            }
        }
    } else {
        // a parameter with more cells than a tile holds: accumulate over chunks
        const int64_t nbatch = (D + dstep - 1) / dstep;
        for (int64_t bt = 0; bt < nbatch; bt++) {
            const int64_t d = bt * dstep + d0;
            CT acc = 0;
            for (int ch = 0; ch < nchunks; ch++) {
                const int c0 = ch * TW;
                const int cn = min(TW, ncell - c0);
                build(c0, cn);
                const int lo = max(pc0, c0) - c0, hi = min(pc1, c0 + cn) - c0;
                if (has_p && d < D && lo < hi) acc += pair_sum(d, lo, hi);
            }
            if (has_p && d < D) {
                if (scale_p) acc = (acc * scale_d[d]) * sp;
                J[d * P + p] = acc;
            }
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

// shared-memory plan: tile width TW (power of two, <= 16) and the cells G
// staged at a time for the given table precision
bool plan(const Context &c, int dtype, int *TW, int *G, int ndip = -1) {
    const size_t uv = 2 * (size_t)c.nK * c.mesh.nv * (c.nE + 1) * sizeof(double);
    const size_t tab = (size_t)c.nK * (ndip < 0 ? c.nA + c.nM : ndip) * c.mesh.nv * (dtype == 0 ? 8 : 4);
    for (size_t budget : {kSmemBudget, kSmemBudgetLarge})
        for (int tw : {16, 8, 4, 2, 1}) {
            if (tw * tab + uv > budget) continue;
            *TW = tw;
            *G = (int)std::max<size_t>(1, std::min<size_t>(4, (budget - tw * tab) / uv));
            return true;
        }
    return false;
}

template <typename CT>
void launch(Context &c, const double *model, CT *J, int dtype, cudaStream_t s) {
    MeshData &m = c.mesh;
    JacTiles &T = c.jtiles[dtype];
    const int ntiles = (int)T.tile_p.size() - 1;
    if (ntiles <= 0) return;
    if (c.nK > 64) throw Error(ERTGB_BAD_INPUT, "Jacobian supports at most 64 wavenumbers");
    const int TW = T.max_cells, G = T.stage_cells;
    const size_t uv = (size_t)c.nK * m.nv * (c.nE + 1);
    const size_t smem = 2 * uv * G * sizeof(double) + (size_t)c.nK * (c.nA + c.nM) * m.nv * TW * sizeof(CT);
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
        if (T.chunks.empty()) {
            ERTGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            kern<<<ntiles, kThreads, smem, s>>>(T.d_tile_p.p, m.d_pcell_ptr.p, m.d_pcell.p, m.d_cells.p, m.d_K.p,
                                                m.d_M.p, c.d_k.p, c.d_w.p, c.nK, c.nE, c.Rpad, c.d_x.p, c.nA,
                                                c.d_dip_a.p, c.nM, c.d_dip_m.p, c.d_data_dip.p, sd, sp, m.P, c.D, G, J);
            ERTGB_CUDA(cudaGetLastError());
            return;
        }
        // data chunks: rows [d0, d1) of J with the chunk's own dipole tables
        for (const auto &ch : T.chunks) {
            const size_t sm = 2 * uv * G * sizeof(double) + (size_t)c.nK * (ch->nA + ch->nM) * m.nv * TW * sizeof(CT);
            ERTGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
            kern<<<ntiles, kThreads, sm, s>>>(T.d_tile_p.p, m.d_pcell_ptr.p, m.d_pcell.p, m.d_cells.p, m.d_K.p,
                                              m.d_M.p, c.d_k.p, c.d_w.p, c.nK, c.nE, c.Rpad, c.d_x.p, ch->nA,
                                              ch->dip_a.p, ch->nM, ch->dip_m.p, ch->data_dip.p,
                                              sd ? sd + ch->d0 : nullptr, sp, m.P, ch->d1 - ch->d0, G,
                                              J + ch->d0 * m.P);
            ERTGB_CUDA(cudaGetLastError());
        }
    };
    auto by_tw = [&](auto nvc) {
        constexpr int NV = decltype(nvc)::value;
        if (TW == 16) go(k_jacobian<NV, CT, 16>);
        else if (TW == 8) go(k_jacobian<NV, CT, 8>);
        else if (TW == 4) go(k_jacobian<NV, CT, 4>);
        else if (TW == 2) go(k_jacobian<NV, CT, 2>);
        else go(k_jacobian<NV, CT, 1>);
    };
    switch (m.nv) {
        case 3: by_tw(std::integral_constant<int, 3>()); break;
        case 4: by_tw(std::integral_constant<int, 4>()); break;
        case 6: by_tw(std::integral_constant<int, 6>()); break;
        default: by_tw(std::integral_constant<int, 10>()); break;
    }
}

}  // namespace

// Contiguous data chunks, each with at most cap distinct current + potential
// dipoles, and their chunk-local dipole tables.
static void build_chunks(Context &c, int cap, JacTiles &T) {
    const std::vector<int32_t> &ab = c.abmn_h;
    int64_t d = 0;
    while (d < c.D) {
        auto ch = std::make_unique<JacChunk>();
        ch->d0 = d;
        std::map<std::pair<int32_t, int32_t>, int32_t> amap, mmap;
        std::vector<int32_t> dip_a, dip_m, data_dip;
        for (; d < c.D; d++) {
            const auto ka = std::make_pair(ab[4 * d], ab[4 * d + 1]);
            const auto km = std::make_pair(ab[4 * d + 2], ab[4 * d + 3]);
            const int add = (amap.count(ka) ? 0 : 1) + (mmap.count(km) ? 0 : 1);
            if ((int)(amap.size() + mmap.size()) + add > cap && d > ch->d0) break;
            auto ia = amap.emplace(ka, (int32_t)amap.size());
            if (ia.second) { dip_a.push_back(ka.first); dip_a.push_back(ka.second); }
            auto im = mmap.emplace(km, (int32_t)mmap.size());
            if (im.second) { dip_m.push_back(km.first); dip_m.push_back(km.second); }
            data_dip.push_back(ia.first->second);
            data_dip.push_back(im.first->second);
        }
        ch->d1 = d;
        ch->nA = (int)amap.size();
        ch->nM = (int)mmap.size();
        ch->dip_a.upload(dip_a, c.stream);
        ch->dip_m.upload(dip_m, c.stream);
        ch->data_dip.upload(data_dip, c.stream);
        T.chunks.push_back(std::move(ch));
    }
}

// Parameter -> cells and the Jacobian tiles of both table precisions
// (consecutive parameters with at most TW cells per tile).
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
    for (int dt = 0; dt < 2; dt++) {
        JacTiles &T = c.jtiles[dt];
        T.tile_p.assign(1, 0);
        T.chunks.clear();
        int TW = 0, G = 0;
        if (!plan(c, dt, &TW, &G)) {
            // split the scheme into data chunks whose distinct dipoles fit
            int cap = 0;
            for (int nd = c.nA + c.nM; nd >= 2; nd = nd * 3 / 4)
                if (plan(c, dt, &TW, &G, nd)) {
                    cap = nd;
                    break;
                }
            if (cap < 2) {
                T.max_cells = 0;
                continue;
            }
            build_chunks(c, cap, T);
        }
        T.max_cells = TW;
        T.stage_cells = G;
        int64_t p = 0;
        while (p < P) {
            int64_t q = p, ncell = 0;
            while (q < P && q - p < TW) {
                const int64_t cq = m.pcell_ptr[q + 1] - m.pcell_ptr[q];
                if (q > p && ncell + cq > TW) break;
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
        throw Error(ERTGB_BAD_INPUT, "Jacobian tables of one cell exceed shared memory "
                                     "(too many wavenumbers x distinct dipoles)");
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
