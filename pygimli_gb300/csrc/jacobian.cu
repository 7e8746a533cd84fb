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
#include <array>
#include <cstring>
#include <map>
#include <set>
#include <type_traits>

#include "ertgb_internal.cuh"

namespace ertgb {

namespace {

constexpr int kThreads = 512;
constexpr size_t kSmemBudget = 110 * 1024;       // two blocks per SM
constexpr size_t kSmemBudgetLarge = 220 * 1024;  // one block per SM (many wavenumbers x dipoles)
constexpr size_t kStiffSmem = 220 * 1024;       // stiffness kernel: two table buffers + staging
constexpr size_t kStiffStage = 24 * 1024;       // stiffness kernel: staging of the producers

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

// ---------------------------------------------------------------------------
// Stiffness-only Jacobian (one wavenumber k = 0, i.e. the 3-D operator, and at
// most one cell per parameter): a bandwidth-bound stream of J rows.
//
// K_c has zero row and column sums (the gradient of a constant vanishes), so
// with the shifted dipole potentials g_j = delta_j - delta_0 (j = 1..nv-1)
//   J[d, c] = delta_ab^T K_c delta_mn = sum_{i>=1} (K_c g_ab)_i g_mn,i .
// The shift removes the cancellation of K_c delta for cells far from a
// dipole, and the sum has nv-1 instead of nv terms.  The FP64 J forms every
// difference and product in FP64.  The FP32 J splits each FP64 potential
// exactly into hi + lo (hi = fl32(u), lo = fl32(u - hi)) once per response and
// forms the differences as (hi_x - hi_y) + (lo_x - lo_y): where the two
// potentials cancel, hi_x - hi_y is exact (Sterbenz), so the result is the
// FP64 difference rounded to FP32 up to 2^-47 of the potentials; products
// and the J store are FP32.
//
// One block per TW-parameter tile (thread = (datum sub-row, parameter)),
// persistent over tiles.  Per data chunk the block builds, in shared memory,
//   TA[ia][slot] = (K_c g_ab)_{1..nv-1}   for every distinct current dipole,
//   TM[im][slot] = g_mn,{1..nv-1}         for every distinct potential dipole,
// then each warp streams a balanced range of the chunk's data (sorted by
// current dipole, so a TA row stays in registers across its group): one table
// row load, nv-1 FMAs and one store per (datum, parameter); a warp writes
// 32 / TW row segments of TW consecutive parameters.
// ---------------------------------------------------------------------------

constexpr int kSJT = 512;    // threads of the stiffness kernel (one block per SM)
constexpr int kSJProd = 4;   // producer warps (tables); the other warps stream J rows
constexpr int kSTW = 16;     // parameters per tile
// named barriers (0 is __syncthreads): buffer full / empty, producers only
constexpr int kBarFull0 = 1, kBarEmpty0 = 3, kBarProd = 5;

__device__ __forceinline__ void named_sync(int id, int n) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}
__device__ __forceinline__ void named_arrive(int id, int n) {
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// chunk descriptor: data range of the sorted list, electrodes, dipoles and
// their offsets into the concatenated lists, cells staged at a time
struct StiffChunk {
    int32_t s0, s1, nEl, nA, nM, off_el, off_a, off_m, G, pad[3];
};
static_assert(sizeof(StiffChunk) == 12 * sizeof(int32_t), "chunk descriptor layout");

template <typename OT> __host__ __device__ constexpr int nvp_of(int nm1) {
    return sizeof(OT) == 4 ? (nm1 + 3) / 4 * 4 : (nm1 + 1) / 2 * 2;
}

// electrode-level staging element: FP32 (hi, lo) difference pair or FP64
template <typename OT> struct StageOf { using type = double; };
template <> struct StageOf<float> { using type = float2; };

__device__ __forceinline__ float stage_diff(float2 x, float2 y) { return (x.x - y.x) + (x.y - y.y); }
__device__ __forceinline__ double stage_diff(double x, double y) { return x - y; }
__device__ __forceinline__ float2 stage_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double stage_sub(double a, double b) { return a - b; }

// one table row of NVP values (NVP * sizeof(OT) a multiple of 16 bytes, rows 16-byte aligned)
template <typename OT, int NVP> __device__ __forceinline__ void load_row(const OT *p, OT *v) {
    static_assert(NVP * sizeof(OT) % 16 == 0, "table rows are whole 16-byte units");
    const int4 *q = reinterpret_cast<const int4 *>(p);
#pragma unroll
    for (int i = 0; i < (int)(NVP * sizeof(OT) / 16); i++) reinterpret_cast<int4 *>(v)[i] = q[i];
}
template <typename OT, int NVP> __device__ __forceinline__ void store_row(OT *p, const OT *v) {
    int4 *q = reinterpret_cast<int4 *>(p);
#pragma unroll
    for (int i = 0; i < (int)(NVP * sizeof(OT) / 16); i++) q[i] = reinterpret_cast<const int4 *>(v)[i];
}

template <int NV, typename OT>
__global__ void __launch_bounds__(kSJT, 1)
    k_jac_stiff(int64_t ntiles, int64_t P, const int32_t *__restrict__ pc, const int32_t *__restrict__ cells,
                const double *__restrict__ K, const typename StageOf<OT>::type *__restrict__ pot, int64_t Rpad,
                const StiffChunk *__restrict__ chunks, int nchunks, int buf_bytes, int G,
                const int32_t *__restrict__ el, const int32_t *__restrict__ dipa, const int32_t *__restrict__ dipm,
                const int4 *__restrict__ meta, const OT *__restrict__ sd, const OT *__restrict__ sp, OT w0,
                OT *__restrict__ J) {
    using ST = typename StageOf<OT>::type;
    constexpr int TW = kSTW;
    constexpr int NM1 = NV - 1;
    constexpr int NVP = nvp_of<OT>(NM1);
    constexpr int SUB = 32 / TW;                  // data rows per warp step
    constexpr int NPT = kSJProd * 32;             // producer threads
    constexpr int NCW = kSJT / 32 - kSJProd;      // consumer warps
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t nitems = ntiles * nchunks;
    // buffer b: [TA | TM] tables, then sps[TW] (w_0 / model^2 per slot), node_s[TW * NV]
    auto buf = [&](int b) { return smem_raw + (size_t)b * buf_bytes; };
    const size_t tab_bytes = (size_t)buf_bytes - TW * sizeof(OT) - TW * NV * sizeof(int32_t);
    ST *Eg = reinterpret_cast<ST *>(smem_raw + 2 * (size_t)buf_bytes);

    if (warp < kSJProd) {
        // ---------------- producers: tables of item i into buffer i & 1
        const int t = threadIdx.x;
        int i = 0;
        for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x, i++) {
            const int b = i & 1;
            if (i >= 2) named_sync(kBarEmpty0 + b, kSJT);  // consumers are done with buffer b
            const int64_t tile = item / nchunks;
            const StiffChunk cd = chunks[item % nchunks];
            const int64_t p0 = tile * TW;
            const int TP = (int)(P - p0 < (int64_t)TW ? P - p0 : (int64_t)TW);
            OT *TA = reinterpret_cast<OT *>(buf(b));
            OT *TM = TA + (size_t)cd.nA * TW * NVP;
            OT *sps = reinterpret_cast<OT *>(buf(b) + tab_bytes);
            int32_t *node_s = reinterpret_cast<int32_t *>(sps + TW);
            OT *Ks = reinterpret_cast<OT *>(Eg + (size_t)G * NM1 * cd.nEl);
            for (int q = t; q < TW * NV; q += NPT) {
                const int g = q / NV, k = q - g * NV;
                const int cell = g < TP ? pc[p0 + g] : -1;
                node_s[q] = cell < 0 ? -1 : cells[(int64_t)cell * NV + k];
            }
            for (int q = t; q < TW; q += NPT) sps[q] = (sp && q < TP) ? w0 * sp[p0 + q] : w0;
            const int32_t *elc = el + cd.off_el;
            const int32_t *dac = dipa + 2 * cd.off_a;
            const int32_t *dmc = dipm + 2 * cd.off_m;
            named_sync(kBarProd, NPT);
            for (int g0 = 0; g0 < TW; g0 += G) {
                const int gn = min(G, TW - g0);
                // electrode-level shifted potentials u_e(node j) - u_e(node 0), j = 1..nv-1
                const int nst = gn * NM1 * cd.nEl;
                for (int q = t; q < nst; q += NPT) {
                    const int e = q % cd.nEl;
                    const int gj = q / cd.nEl;  // g * NM1 + (j - 1)
                    const int g = gj / NM1, j = gj - g * NM1 + 1;
                    const int n0 = node_s[(g0 + g) * NV], nj = node_s[(g0 + g) * NV + j];
                    const int ge = elc[e];
                    ST v{};
                    if (n0 >= 0 && ge >= 0) v = stage_sub(pot[(int64_t)nj * Rpad + ge], pot[(int64_t)n0 * Rpad + ge]);
                    Eg[q] = v;
                }
                for (int q = t; q < gn * NM1 * NM1; q += NPT) {
                    const int g = q / (NM1 * NM1), ij = q - g * NM1 * NM1;
                    const int r = ij / NM1 + 1, j = ij % NM1 + 1;
                    const int cell = (g0 + g) < TP ? pc[p0 + g0 + g] : -1;
                    Ks[q] = cell < 0 ? (OT)0 : (OT)K[(int64_t)cell * NV * NV + r * NV + j];
                }
                named_sync(kBarProd, NPT);
                // TA rows (w_0 / model^2 * K_c g_ab) and TM rows (g_mn) of the staged cells
                for (int q = t; q < (cd.nA + cd.nM) * gn; q += NPT) {
                    const int g = q % gn;
                    int dp = q / gn;
                    const bool isA = dp < cd.nA;
                    if (!isA) dp -= cd.nA;
                    const int32_t *dd = isA ? dac : dmc;
                    const int a = dd[2 * dp], bb = dd[2 * dp + 1];
                    const ST *Ea = Eg + (size_t)g * NM1 * cd.nEl;
                    OT gv[NM1];
#pragma unroll
                    for (int j = 0; j < NM1; j++) gv[j] = (OT)stage_diff(Ea[j * cd.nEl + a], Ea[j * cd.nEl + bb]);
                    OT out[NVP];
                    if (isA) {
                        const OT *Kg = Ks + (size_t)g * NM1 * NM1;
                        const OT f = sps[g0 + g];
#pragma unroll
                        for (int r = 0; r < NM1; r++) {
                            OT s = 0;
#pragma unroll
                            for (int j = 0; j < NM1; j++) s = fma(Kg[r * NM1 + j], gv[j], s);
                            out[r] = s * f;
                        }
                    } else {
#pragma unroll
                        for (int r = 0; r < NM1; r++) out[r] = gv[r];
                    }
#pragma unroll
                    for (int r = NM1; r < NVP; r++) out[r] = 0;
                    store_row<OT, NVP>((isA ? TA : TM) + ((size_t)dp * TW + g0 + g) * NVP, out);
                }
                named_sync(kBarProd, NPT);  // Eg / Ks reused by the next cells
            }
            __threadfence_block();
            named_arrive(kBarFull0 + b, kSJT);
        }
        // match the consumers' releases of the last two items
        for (int k = (i >= 2 ? i - 2 : 0); k < i; k++) named_sync(kBarEmpty0 + (k & 1), kSJT);
    } else {
        // ---------------- consumers: stream the J rows of item i from buffer i & 1
        const int cw = warp - kSJProd;
        const int slot = lane % TW, sub = lane / TW;
        int i = 0;
        for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x, i++) {
            const int b = i & 1;
            named_sync(kBarFull0 + b, kSJT);
            const int64_t tile = item / nchunks;
            const StiffChunk cd = chunks[item % nchunks];
            const int64_t p0 = tile * TW;
            const int TP = (int)(P - p0 < (int64_t)TW ? P - p0 : (int64_t)TW);
            const OT *TA = reinterpret_cast<const OT *>(buf(b));
            const OT *TM = TA + (size_t)cd.nA * TW * NVP;
            // consumer warp cw streams a balanced range of the chunk's data; per
            // batch of 32 data one coalesced load of their (datum, dipoles) and
            // scale, broadcast by shuffles; the SUB lane groups of a warp take
            // consecutive data of the batch
            const int len = cd.s1 - cd.s0;
            const int sb = cd.s0 + (int)((int64_t)len * cw / NCW);
            const int se = cd.s0 + (int)((int64_t)len * (cw + 1) / NCW);
            int cur = -1;
            OT ta[NVP];
#pragma unroll
            for (int r = 0; r < NVP; r++) ta[r] = 0;
            for (int base = sb; base < se; base += 32) {
                const int sl = base + lane;
                int4 mm = make_int4(0, 0, 0, 0);
                OT sdl = (OT)1;
                if (sl < se) {
                    mm = meta[sl];
                    if (sd) sdl = sd[mm.x];
                }
#pragma unroll 4
                for (int k = 0; k < 32 / SUB; k++) {
                    const int src = k * SUB + sub;
                    const int dm = __shfl_sync(0xffffffffu, mm.x, src);
                    const int ia = __shfl_sync(0xffffffffu, mm.y, src);
                    const int im = __shfl_sync(0xffffffffu, mm.z, src);
                    const OT sdk = __shfl_sync(0xffffffffu, sdl, src);
                    if (base + src >= se) continue;
                    if (ia != cur) {
                        cur = ia;
                        load_row<OT, NVP>(TA + ((size_t)cur * TW + slot) * NVP, ta);
                    }
                    OT tm[NVP];
                    load_row<OT, NVP>(TM + ((size_t)im * TW + slot) * NVP, tm);
                    OT acc = 0;
#pragma unroll
                    for (int r = 0; r < NM1; r++) acc = fma(ta[r], tm[r], acc);
                    if (slot < TP) J[(int64_t)dm * P + p0 + slot] = acc * sdk;
                }
            }
            named_arrive(kBarEmpty0 + b, kSJT);
        }
    }
}

// FP64 potentials -> exact (hi, lo) FP32 pairs
__global__ void k_split_hilo(int64_t total, const double *__restrict__ x, float2 *__restrict__ y) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const double v = x[t];
        const float h = (float)v;
        y[t] = make_float2(h, (float)(v - (double)h));
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
void launch_stiff(Context &c, const CT *sd, const CT *sp, CT *J, int dtype, cudaStream_t s) {
    using ST = typename StageOf<CT>::type;
    MeshData &m = c.mesh;
    JacStiff &S = c.jstiff[dtype];
    const ST *pot = reinterpret_cast<const ST *>(c.d_x.p);
    if (dtype == 1) {
        const int64_t total = m.n * c.Rpad;
        c.d_xhl.alloc((size_t)total);
        k_split_hilo<<<(unsigned)std::min<int64_t>(ceil_div(total, 256), 8192), 256, 0, s>>>(total, c.d_x.p,
                                                                                            c.d_xhl.p);
        ERTGB_CUDA(cudaGetLastError());
        pot = reinterpret_cast<const ST *>(c.d_xhl.p);
    }
    int nsm = 0;
    ERTGB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c.device));
    const CT w0 = (CT)c.w[0];
    auto go = [&](auto kern) {
        ERTGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S.smem));
        const int64_t grid = std::min<int64_t>(S.ntiles * S.nchunks, (int64_t)nsm);
        kern<<<(unsigned)grid, kSJT, S.smem, s>>>(S.ntiles, m.P, S.d_pc.p, m.d_cells.p, m.d_K.p, pot, c.Rpad,
                                                  reinterpret_cast<const StiffChunk *>(S.d_chunks.p), S.nchunks,
                                                  (int)S.buf_bytes, S.G, S.d_el.p, S.d_dipa.p, S.d_dipm.p,
                                                  reinterpret_cast<const int4 *>(S.d_meta.p), sd, sp, w0, J);
        ERTGB_CUDA(cudaGetLastError());
    };
    auto by_tw = [&](auto nvc) {
        constexpr int NV = decltype(nvc)::value;
        go(k_jac_stiff<NV, CT>);
    };
    switch (m.nv) {
        case 3: by_tw(std::integral_constant<int, 3>()); break;
        case 4: by_tw(std::integral_constant<int, 4>()); break;
        case 6: by_tw(std::integral_constant<int, 6>()); break;
        default: by_tw(std::integral_constant<int, 10>()); break;
    }
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
    if (c.jstiff[dtype].ok) {
        launch_stiff<CT>(c, sd, sp, J, dtype, s);
        return;
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

// Plan of the stiffness kernel for one J precision (dt 0: FP64, 1: FP32).
// Applies with one wavenumber k = 0 (3-D) and at most one cell per parameter.
// Shared memory: two table buffers (tables of one data chunk for a tile of
// kSTW parameters, the slot scales and the tile's cell nodes) and the
// producers' staging of G cells.  Data are split into contiguous chunks whose
// tables fit one buffer and whose electrodes fit the staging with G >= 2.
static void build_stiff_plan(Context &c, int dt) {
    JacStiff &S = c.jstiff[dt];
    S.ok = false;
    MeshData &m = c.mesh;
    if (c.nK != 1 || c.k[0] != 0.0 || c.D == 0 || m.P == 0) return;
    if (m.nv != 3 && m.nv != 4 && m.nv != 6 && m.nv != 10) return;
    std::vector<int32_t> pc((size_t)m.P, -1);
    for (int64_t p = 0; p < m.P; p++) {
        const int32_t cnt = m.pcell_ptr[p + 1] - m.pcell_ptr[p];
        if (cnt > 1) return;
        if (cnt == 1) pc[p] = m.pcell[m.pcell_ptr[p]];
    }
    const int TW = kSTW;
    const int nm1 = m.nv - 1;
    const size_t sz = dt == 0 ? 8 : 4;
    const size_t nvp = dt == 0 ? (nm1 + 1) / 2 * 2 : (nm1 + 3) / 4 * 4;
    const size_t per_dip = (size_t)TW * nvp * sz;                   // table bytes per dipole
    const size_t fixed = (size_t)TW * sz + (size_t)TW * m.nv * 4;   // slot scales + cell nodes
    const size_t per_el = (size_t)nm1 * 8;                          // staging bytes per electrode and cell
    const size_t ks = (size_t)nm1 * nm1 * sz;                       // staging of K per cell
    const int el_cap = (int)((kStiffStage / 2 - ks) / per_el);      // G >= 2
    const size_t tab_cap = ((kStiffSmem - kStiffStage) / 2 - fixed) / 16 * 16;
    const std::vector<int32_t> &ab = c.abmn_h;
    std::vector<StiffChunk> chunks;
    std::vector<int32_t> el, dipa, dipm;
    std::vector<int4> meta;
    meta.reserve((size_t)c.D);
    size_t tab_max = 0;
    int el_max = 0;
    int64_t d = 0;
    while (d < c.D) {
        std::map<int32_t, int32_t> emap;
        std::map<std::pair<int32_t, int32_t>, int32_t> amap, mmap;
        std::vector<std::array<int32_t, 3>> rows;  // (ia, d, im) of the chunk
        const int64_t d0 = d;
        for (; d < c.D; d++) {
            const int32_t *q = &ab[4 * d];
            std::set<int32_t> newe;
            for (int i = 0; i < 4; i++)
                if (!emap.count(q[i])) newe.insert(q[i]);
            const int ne = (int)(emap.size() + newe.size());
            const int na = (int)amap.size() + (amap.count({q[0], q[1]}) ? 0 : 1);
            const int nmm = (int)mmap.size() + (mmap.count({q[2], q[3]}) ? 0 : 1);
            if ((size_t)(na + nmm) * per_dip > tab_cap || ne > el_cap) {
                if (d == d0) return;  // one datum does not fit: no plan
                break;
            }
            for (int i = 0; i < 4; i++) emap.emplace(q[i], (int32_t)emap.size());
            const int32_t ia = amap.emplace(std::make_pair(q[0], q[1]), (int32_t)amap.size()).first->second;
            const int32_t im = mmap.emplace(std::make_pair(q[2], q[3]), (int32_t)mmap.size()).first->second;
            rows.push_back({ia, (int32_t)d, im});
        }
        StiffChunk cd{};
        cd.s0 = (int32_t)meta.size();
        cd.s1 = cd.s0 + (int32_t)rows.size();
        cd.nEl = (int32_t)emap.size();
        cd.nA = (int32_t)amap.size();
        cd.nM = (int32_t)mmap.size();
        cd.off_el = (int32_t)el.size();
        cd.off_a = (int32_t)(dipa.size() / 2);
        cd.off_m = (int32_t)(dipm.size() / 2);
        tab_max = std::max(tab_max, (size_t)(cd.nA + cd.nM) * per_dip);
        el_max = std::max(el_max, cd.nEl);
        std::vector<int32_t> eloc(emap.size());
        for (auto &kv : emap) eloc[kv.second] = kv.first;
        el.insert(el.end(), eloc.begin(), eloc.end());
        std::vector<int32_t> da(2 * amap.size()), dm(2 * mmap.size());
        for (auto &kv : amap) {
            da[2 * kv.second] = emap[kv.first.first];
            da[2 * kv.second + 1] = emap[kv.first.second];
        }
        for (auto &kv : mmap) {
            dm[2 * kv.second] = emap[kv.first.first];
            dm[2 * kv.second + 1] = emap[kv.first.second];
        }
        dipa.insert(dipa.end(), da.begin(), da.end());
        dipm.insert(dipm.end(), dm.begin(), dm.end());
        std::sort(rows.begin(), rows.end());
        for (auto &r : rows) meta.push_back(make_int4(r[1], r[0], r[2], 0));
        chunks.push_back(cd);
    }
    const size_t per_cell = (size_t)el_max * per_el + ks;
    S.G = (int)std::max<size_t>(2, std::min<size_t>(8, kStiffStage / per_cell));
    S.buf_bytes = (tab_max + 15) / 16 * 16 + fixed;
    S.smem = 2 * S.buf_bytes + (size_t)S.G * per_cell;
    S.ntiles = ceil_div(m.P, TW);
    S.nchunks = (int)chunks.size();
    S.d_pc.upload(pc, c.stream);
    S.d_el.upload(el, c.stream);
    S.d_dipa.upload(dipa, c.stream);
    S.d_dipm.upload(dipm, c.stream);
    std::vector<int32_t> cw(chunks.size() * 12);
    std::memcpy(cw.data(), chunks.data(), cw.size() * sizeof(int32_t));
    S.d_chunks.upload(cw, c.stream);
    std::vector<int32_t> mw(meta.size() * 4);
    std::memcpy(mw.data(), meta.data(), mw.size() * sizeof(int32_t));
    S.d_meta.upload(mw, c.stream);
    S.ok = true;
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
    for (int dt = 0; dt < 2; dt++) build_stiff_plan(c, dt);
}

void jacobian(Context &c, const double *model, int n_model, void *J, int dtype, cudaStream_t s) {
    if (c.jtiles[dtype].max_cells == 0 && !c.jstiff[dtype].ok)
        throw Error(ERTGB_BAD_INPUT, "Jacobian tables of one cell exceed shared memory "
                                     "(too many wavenumbers x distinct dipoles)");
    const double *mdl = (n_model == c.mesh.P) ? model : nullptr;
    if (dtype == 0) launch<double>(c, mdl, (double *)J, 0, s);
    else launch<float>(c, mdl, (float *)J, 1, s);
}

void profile_jacobian(Context &c, int reps, void *J, int dtype, double *ms, double *bytes, double *flops) {
    if (!c.have_pot) throw Error(ERTGB_STATE, "profile needs a completed response");
    if (c.jtiles[dtype].max_cells == 0 && !c.jstiff[dtype].ok)
        throw Error(ERTGB_BAD_INPUT, "no Jacobian plan for this scheme");
    MeshData &m = c.mesh;
    cudaStream_t s = c.stream;
    auto once = [&] {
        if (dtype == 0) launch<double>(c, nullptr, (double *)J, 0, s);
        else launch<float>(c, nullptr, (float *)J, 1, s);
    };
    once();
    ERTGB_CUDA(cudaEventRecord(c.ev[0], s));
    for (int r = 0; r < reps; r++) once();
    ERTGB_CUDA(cudaEventRecord(c.ev[1], s));
    ERTGB_CUDA(cudaEventSynchronize(c.ev[1]));
    float t = 0.f;
    ERTGB_CUDA(cudaEventElapsedTime(&t, c.ev[0], c.ev[1]));
    *ms = (double)t / reps;
    const double Ca = (double)m.pcell.size();
    const double sJ = dtype == 0 ? 8.0 : 4.0;
    // J written once, potentials read once, cell nodes + element matrices,
    // parameter->cell map, scheme and its dipole indices
    *bytes = (double)c.D * m.P * sJ + (double)m.n * c.Rpad * 8.0 + Ca * (m.nv * 4.0 + 2.0 * m.nv * m.nv * 8.0 + 4.0) +
             (double)(m.P + 1) * 4.0 + (double)c.D * (8.0 + 8.0) + (double)(c.nA + c.nM) * 8.0;
    if (c.jstiff[dtype].ok) {
        // stiffness plan: shifted differences per electrode and dipole, K g per
        // current dipole, nv-1 FMAs per (datum, cell)
        const int nm1 = m.nv - 1;
        *flops = Ca * ((c.nE + 1) * nm1 + (c.nA + c.nM) * nm1 * 3.0 + c.nA * 2.0 * nm1 * nm1) +
                 (double)c.D * Ca * (2.0 * nm1 + 2.0);
    } else {
        // V = S U, the dipole differences, and one nv-term dot per (datum, cell, k)
        *flops = Ca * c.nK * ((c.nE + 1) * m.nv * 2.0 * m.nv + (c.nA + c.nM) * m.nv) +
                 (double)c.D * Ca * c.nK * (m.nv * 2.0 + 2.0);
    }
}

}  // namespace ertgb
