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
constexpr size_t kStiffSmem = 226 * 1024;      // stiffness kernel: one block per SM (227 KB max)

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
// forms the four-potential differences as
//   ((hi_a,j - hi_a,0) - (hi_b,j - hi_b,0)) + ((lo_a,j - lo_a,0) - (lo_b,j - lo_b,0)):
// where potentials cancel the hi differences are exact (Sterbenz), so the
// result is the FP64 difference rounded to FP32 up to 2^-47 of the
// potentials; products and the J store are FP32.
//
// One block of 1024 threads per SM, persistent over tiles of 32 parameters.
// Per tile the block copies the potential rows of the tile's distinct nodes
// into shared memory with asynchronous 16-byte copies (cp.async; a tile of 32
// tetrahedra has at most ~30 distinct nodes against 128 cell nodes), once for
// every data chunk.  Per data chunk it then builds the tables
//   TA[ia] = w_0 / model^2 * (K_c g_ab)_{1..nv-1}  for every distinct current dipole,
//   TM[im] = g_mn,{1..nv-1}                        for every distinct potential dipole,
// each row component-major with the 32 slots fastest, and streams the chunk's
// data: every warp takes a balanced range of the data records (datum,
// ia | im << 16, geometric factor), sorted by current dipole so a lane's TA
// values stay in registers across a group, staged 16 at a time in shared
// memory with the next batch loaded ahead; 16 lanes per record, each lane two
// adjacent parameters: nv-1 conflict-free 8-byte table loads, 2(nv-1) FMAs and
// one 8-byte J store (two 4-byte stores when P is odd).
// ---------------------------------------------------------------------------

constexpr int kSJT = 1024;  // threads of the stiffness kernel (one block per SM)
constexpr int kSTW = 32;    // parameters per tile
constexpr int kNREC = 16;   // data records staged per warp batch

// chunk descriptor: data range of the sorted records, dipoles and their offsets
struct StiffChunk {
    int32_t s0, s1, nA, nM, off_a, off_m, pad[6];
};
static_assert(sizeof(StiffChunk) == 12 * sizeof(int32_t), "chunk descriptor layout");

// two adjacent slots of a table component (one 8- or 16-byte access)
template <typename OT> struct Pair { using type = double2; };
template <> struct Pair<float> { using type = float2; };

// staged potential element: FP32 (hi, lo) pair or FP64
template <typename OT> struct StageOf { using type = double; };
template <> struct StageOf<float> { using type = float2; };

// (x_j - x_0) - (y_j - y_0) for the hi and the lo parts, summed
__device__ __forceinline__ float dipole_shift(float2 xj, float2 x0, float2 yj, float2 y0) {
    return ((xj.x - x0.x) - (yj.x - y0.x)) + ((xj.y - x0.y) - (yj.y - y0.y));
}
__device__ __forceinline__ double dipole_shift(double xj, double x0, double yj, double y0) {
    return (xj - x0) - (yj - y0);
}

// per-datum scale (the geometric factor) carried in a data record: FP32 in .z, FP64 in (.z, .w)
template <typename OT> __device__ __forceinline__ OT record_scale(int4 m);
template <> __device__ __forceinline__ float record_scale<float>(int4 m) { return __int_as_float(m.z); }
template <> __device__ __forceinline__ double record_scale<double>(int4 m) {
    return __hiloint2double(m.w, m.z);
}

// asynchronous 16-byte global -> shared copy (both addresses 16-byte aligned)
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;" ::: "memory");
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// VEC: 4 = four adjacent parameters per lane and 16-byte stores (FP32 J with
// a row length and base aligned to four), 2 = two per lane and paired
// stores, 1 = two per lane, element stores
template <int NV, typename OT, int VEC>
__global__ void __launch_bounds__(kSJT, 1)
    k_jac_stiff(int64_t ntiles, int64_t P, const int32_t *__restrict__ pc, const double *__restrict__ K,
                const typename StageOf<OT>::type *__restrict__ pot, int64_t Rpad, int nE, int RS,
                const int32_t *__restrict__ tile_nptr, const int32_t *__restrict__ tnodes,
                const uint8_t *__restrict__ lidx, const StiffChunk *__restrict__ chunks, int nchunks,
                int tab_bytes, int stage_bytes, const int32_t *__restrict__ dipa, const int32_t *__restrict__ dipm,
                const int4 *__restrict__ meta, int scale_data, const OT *__restrict__ sp, OT w0,
                OT *__restrict__ J) {
    using ST = typename StageOf<OT>::type;
    using OT2 = typename Pair<OT>::type;
    constexpr int TW = kSTW;
    constexpr int NM1 = NV - 1;
    constexpr int NW = kSJT / 32;      // warps = data streams
    constexpr int PPL = VEC == 4 ? 4 : 2;  // adjacent parameters (slots) per lane
    constexpr int LPR = TW / PPL;      // lanes per record
    constexpr int RPW = 32 / LPR;      // records per warp step
    static_assert(VEC != 4 || sizeof(OT) == 4, "16-byte stores of four FP32 values");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // [TA | TM tables: row = NM1 x TW values, slot fastest][staged rows Us]
    // [Ks: TW x NM1^2][sps: TW][lid: TW x NV bytes][records: NW x kNREC x (scale, datum, dipoles)]
    OT *tabs = reinterpret_cast<OT *>(smem_raw);
    ST *Us = reinterpret_cast<ST *>(smem_raw + tab_bytes);
    OT *Ks = reinterpret_cast<OT *>(smem_raw + tab_bytes + stage_bytes);
    OT *sps = Ks + TW * NM1 * NM1;
    uint8_t *lid = reinterpret_cast<uint8_t *>(sps + TW);
    OT *rec_f = reinterpret_cast<OT *>(lid + TW * NV);
    int32_t *rec_d = reinterpret_cast<int32_t *>(rec_f + NW * kNREC);
    int32_t *rec_p = rec_d + NW * kNREC;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int s2 = PPL * (lane % LPR), sub = lane / LPR;  // pair phase: slots s2 .. s2 + PPL - 1 of record sub
    const int nE2 = nE & ~1;  // columns copied in 16-byte units
    const int P32 = (int)P;   // parameters < 2^31: 32 x 32 -> 64-bit row offsets

    // shifted dipole potentials g_j = (u_a - u_b)(node j) - (u_a - u_b)(node 0), j = 1..nv-1,
    // of the cell in slot g; false for an empty slot
    auto shifted = [&](int g, int a, int b, OT *gv) -> bool {
        const int l0 = lid[g * NV];
        if (l0 == 0xff) return false;
        const ST *U0 = Us + (size_t)l0 * RS;
        const ST a0 = U0[a], b0 = U0[b];
#pragma unroll
        for (int j = 0; j < NM1; j++) {
            const ST *Uj = Us + (size_t)lid[g * NV + j + 1] * RS;
            gv[j] = (OT)dipole_shift(Uj[a], a0, Uj[b], b0);
        }
        return true;
    };

    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t p0 = tile * TW;
        const int TP = (int)(P - p0 < (int64_t)TW ? P - p0 : (int64_t)TW);
        const int n0 = tile_nptr[tile], nn = tile_nptr[tile + 1] - n0;
        __syncthreads();  // the previous tile is done with every shared buffer
        // the tile's node rows: columns [0, nE2) by 16-byte copies, an odd last column by a
        // plain load, column nE (the electrode at infinity) zero
        {
            const int per = nE2 / 2;
            for (int q = threadIdx.x; q < nn * per; q += kSJT) {
                const int i = q / per, c2 = 2 * (q - i * per);
                cp_async16(Us + (size_t)i * RS + c2, pot + (int64_t)tnodes[n0 + i] * Rpad + c2);
            }
            for (int i = threadIdx.x; i < nn; i += kSJT) {
                if (nE2 < nE) Us[(size_t)i * RS + nE2] = pot[(int64_t)tnodes[n0 + i] * Rpad + nE2];
                Us[(size_t)i * RS + nE] = ST{};
            }
        }
        for (int q = threadIdx.x; q < TW * NV; q += kSJT) lid[q] = lidx[tile * TW * NV + q];
        for (int q = threadIdx.x; q < TW; q += kSJT) sps[q] = (sp && q < TP) ? w0 * sp[p0 + q] : w0;
        for (int q = threadIdx.x; q < TW * NM1 * NM1; q += kSJT) {
            const int g = q / (NM1 * NM1), ij = q - g * NM1 * NM1;
            const int r = ij / NM1 + 1, j = ij % NM1 + 1;
            const int cell = g < TP ? pc[p0 + g] : -1;
            Ks[q] = cell < 0 ? (OT)0 : (OT)K[(int64_t)cell * NV * NV + r * NV + j];
        }
        cp_async_wait_all();
        for (int ch = 0; ch < nchunks; ch++) {
            const StiffChunk cd = chunks[ch];
            const int32_t *dac = dipa + 2 * cd.off_a;
            const int32_t *dmc = dipm + 2 * cd.off_m;
            OT *TA = tabs;
            OT *TM = tabs + (size_t)cd.nA * NM1 * TW;
            __syncthreads();  // staged rows, lid, sps, Ks visible; the previous chunk's pair phase is done
            // TA rows (w_0 / model^2 * K_c g_ab) and TM rows (g_mn) of the chunk's dipoles:
            // thread = (dipole, slot), slot fastest
            for (int q = threadIdx.x; q < (cd.nA + cd.nM) * TW; q += kSJT) {
                const int g = q % TW;
                int dp = q / TW;
                const bool isA = dp < cd.nA;
                if (!isA) dp -= cd.nA;
                const int32_t *dd = isA ? dac : dmc;
                OT gv[NM1], out[NM1];
                const bool ok = shifted(g, dd[2 * dp], dd[2 * dp + 1], gv);
                if (isA) {
                    const OT *Kg = Ks + (size_t)g * NM1 * NM1;
                    const OT f = sps[g];
#pragma unroll
                    for (int i = 0; i < NM1; i++) {
                        OT sacc = 0;
#pragma unroll
                        for (int j = 0; j < NM1; j++) sacc = fma(Kg[i * NM1 + j], gv[j], sacc);
                        out[i] = ok ? sacc * f : (OT)0;
                    }
                } else {
#pragma unroll
                    for (int i = 0; i < NM1; i++) out[i] = ok ? gv[i] : (OT)0;
                }
                OT *dst = (isA ? TA : TM) + (size_t)dp * NM1 * TW + g;
#pragma unroll
                for (int i = 0; i < NM1; i++) dst[i * TW] = out[i];
            }
            __syncthreads();
            // pair phase: warp w streams a balanced range of the chunk's records (sorted by
            // current dipole, so a lane's TA values stay in registers across a group), staged
            // kNREC at a time with the next batch loaded ahead; RPW lane groups take
            // consecutive records, each lane two adjacent parameters
            const int len = cd.s1 - cd.s0;
            const int sb = cd.s0 + (int)((int64_t)len * warp / NW);
            const int se = cd.s0 + (int)((int64_t)len * (warp + 1) / NW);
            const bool st0 = s2 < TP, st1 = s2 + 1 < TP, stall = s2 + PPL - 1 < TP;
            const int tm0 = cd.nA * NM1 * TW + s2;  // element offset of this lane's TM slots
            OT *Jt = J + p0 + s2;
            OT *rf = rec_f + warp * kNREC;
            int32_t *rdd = rec_d + warp * kNREC, *rpp = rec_p + warp * kNREC;
            int cur = -1;
            OT ta[NM1][PPL];
#pragma unroll
            for (int i = 0; i < NM1; i++)
#pragma unroll
                for (int q = 0; q < PPL; q++) ta[i][q] = (OT)0;
            int4 nxt = make_int4(0, 0, 0, 0);
            if (lane < kNREC && sb + lane < se) nxt = meta[sb + lane];
            for (int base = sb; base < se; base += kNREC) {
                __syncwarp();
                if (lane < kNREC) {
                    rdd[lane] = nxt.x;
                    rpp[lane] = nxt.y;
                    rf[lane] = record_scale<OT>(nxt);
                }
                __syncwarp();
                if (lane < kNREC && base + kNREC + lane < se) nxt = meta[base + kNREC + lane];
                const int cnt = min(kNREC, se - base);  // warp-uniform
#pragma unroll
                for (int kk = 0; kk < kNREC / RPW; kk++) {
                    const int k = RPW * kk + sub;
                    if (k >= cnt) break;
                    const int pk = rpp[k];
                    const int ia = pk & 0xffff, im = pk >> 16;
                    if (__builtin_expect(ia != cur, 0)) {
                        cur = ia;
#pragma unroll
                        for (int i = 0; i < NM1; i++) {
                            const OT *src = TA + s2 + (cur * NM1 + i) * TW;
                            if constexpr (VEC == 4) {
                                const float4 v = *reinterpret_cast<const float4 *>(src);
                                ta[i][0] = v.x;
                                ta[i][1] = v.y;
                                ta[i][2] = v.z;
                                ta[i][3] = v.w;
                            } else {
                                const OT2 v = *reinterpret_cast<const OT2 *>(src);
                                ta[i][0] = v.x;
                                ta[i][1] = v.y;
                            }
                        }
                    }
                    const int o = tm0 + im * (NM1 * TW);
                    OT acc[PPL];
#pragma unroll
                    for (int q = 0; q < PPL; q++) acc[q] = (OT)0;
#pragma unroll
                    for (int i = 0; i < NM1; i++) {
                        if constexpr (VEC == 4) {
                            const float4 t = *reinterpret_cast<const float4 *>(tabs + o + i * TW);
                            acc[0] = fma(ta[i][0], t.x, acc[0]);
                            acc[1] = fma(ta[i][1], t.y, acc[1]);
                            acc[2] = fma(ta[i][2], t.z, acc[2]);
                            acc[3] = fma(ta[i][3], t.w, acc[3]);
                        } else {
                            const OT2 t = *reinterpret_cast<const OT2 *>(tabs + o + i * TW);
                            acc[0] = fma(ta[i][0], t.x, acc[0]);
                            acc[1] = fma(ta[i][1], t.y, acc[1]);
                        }
                    }
                    if (scale_data) {
                        const OT f = rf[k];
#pragma unroll
                        for (int q = 0; q < PPL; q++) acc[q] *= f;
                    }
                    OT *dst = Jt + (int64_t)rdd[k] * P32;
                    if constexpr (VEC == 4) {
                        if (stall) {
                            *reinterpret_cast<float4 *>(dst) = make_float4(acc[0], acc[1], acc[2], acc[3]);
                        } else {
#pragma unroll
                            for (int q = 0; q < PPL; q++)
                                if (s2 + q < TP) dst[q] = acc[q];
                        }
                    } else if (VEC == 2 && st1) {
                        *reinterpret_cast<OT2 *>(dst) = OT2{acc[0], acc[1]};
                    } else {
                        if (st0) dst[0] = acc[0];
                        if (st1) dst[1] = acc[1];
                    }
                }
            }
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
void launch_stiff(Context &c, bool scaled, const CT *sp, CT *J, int dtype, cudaStream_t s) {
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
        const int64_t grid = std::min<int64_t>(S.ntiles, (int64_t)nsm);
        kern<<<(unsigned)grid, kSJT, S.smem, s>>>(
            S.ntiles, m.P, S.d_pc.p, m.d_K.p, pot, c.Rpad, c.nE, S.RS, S.d_nptr.p, S.d_tnodes.p, S.d_lidx.p,
            reinterpret_cast<const StiffChunk *>(S.d_chunks.p), S.nchunks, (int)S.tab_bytes, (int)S.stage_bytes,
            S.d_dipa.p, S.d_dipm.p, reinterpret_cast<const int4 *>(S.d_meta.p), scaled ? 1 : 0, sp, w0, J);
        ERTGB_CUDA(cudaGetLastError());
    };
    // 16-byte stores (FP32) when every row's group of four parameters starts on a
    // four-element boundary, else paired stores on a two-element boundary
    const bool v2 = m.P % 2 == 0 && reinterpret_cast<uintptr_t>(J) % (2 * sizeof(CT)) == 0;
    const bool v4 = sizeof(CT) == 4 && m.P % 4 == 0 && reinterpret_cast<uintptr_t>(J) % 16 == 0;
    auto by_tw = [&](auto nvc) {
        constexpr int NV = decltype(nvc)::value;
        if constexpr (sizeof(CT) == 4 && NV <= 6) {  // 4 (NV - 1) TA registers: spills past NV = 6
            if (v4) {
                go(k_jac_stiff<NV, CT, 4>);
                return;
            }
        }
        if (v2) go(k_jac_stiff<NV, CT, 2>);
        else go(k_jac_stiff<NV, CT, 1>);
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
        launch_stiff<CT>(c, sd != nullptr, sp, J, dtype, s);
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
// Shared memory of one block (one per SM): the potential rows of the tile's
// distinct nodes (staged once per tile), the TA and TM tables of one data chunk, the
// tile's K blocks, slot scales and local node indices, and the warps' record
// batches.  Data are split into contiguous chunks whose dipoles fit the
// table space left by the staging.
static void build_stiff_plan(Context &c, int dt) {
    JacStiff &S = c.jstiff[dt];
    S.ok = false;
    MeshData &m = c.mesh;
    if (c.nK != 1 || c.k[0] != 0.0 || c.D == 0 || m.P == 0 || m.P > INT32_MAX) return;
    if (m.nv != 3 && m.nv != 4 && m.nv != 6 && m.nv != 10) return;
    if ((int64_t)c.kfac_h.size() != c.D) return;
    std::vector<int32_t> pc((size_t)m.P, -1);
    for (int64_t p = 0; p < m.P; p++) {
        const int32_t cnt = m.pcell_ptr[p + 1] - m.pcell_ptr[p];
        if (cnt > 1) return;
        if (cnt == 1) pc[p] = m.pcell[m.pcell_ptr[p]];
    }
    const int TW = kSTW, NV = m.nv;
    const int nm1 = NV - 1;
    const size_t sz = dt == 0 ? 8 : 4;
    const size_t per_dip = (size_t)TW * nm1 * sz;  // table bytes per dipole
    const int RS = (c.nE + 2) / 2 * 2;             // staged row: nE columns + the zero column, even
    const size_t row_bytes = (size_t)RS * 8;
    const size_t fixed = (size_t)TW * nm1 * nm1 * sz + (size_t)TW * sz + (size_t)TW * NV +
                         (size_t)(kSJT / 32) * kNREC * (sz + 8);
    // distinct nodes of every tile and the local index of each (slot, cell node)
    S.ntiles = ceil_div(m.P, TW);
    std::vector<int32_t> nptr(1, 0), tnodes;
    std::vector<uint8_t> lidx((size_t)S.ntiles * TW * NV, 0xff);
    int nl_tile = 0;
    for (int64_t t = 0; t < S.ntiles; t++) {
        std::vector<int32_t> v;
        for (int g = 0; g < TW && t * TW + g < m.P; g++) {
            const int32_t cell = pc[t * TW + g];
            if (cell >= 0) v.insert(v.end(), &m.cells[(size_t)cell * NV], &m.cells[(size_t)cell * NV] + NV);
        }
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        if (v.size() > 254) return;  // 0xff marks an empty slot
        for (int g = 0; g < TW && t * TW + g < m.P; g++) {
            const int32_t cell = pc[t * TW + g];
            if (cell < 0) continue;
            for (int k = 0; k < NV; k++)
                lidx[((size_t)t * TW + g) * NV + k] = (uint8_t)(
                    std::lower_bound(v.begin(), v.end(), m.cells[(size_t)cell * NV + k]) - v.begin());
        }
        nl_tile = std::max(nl_tile, (int)v.size());
        tnodes.insert(tnodes.end(), v.begin(), v.end());
        nptr.push_back((int32_t)tnodes.size());
    }
    const size_t stage = (size_t)nl_tile * row_bytes;
    if (kStiffSmem < fixed + stage + 2 * per_dip) return;
    const size_t tab_cap = (kStiffSmem - fixed - stage) / 16 * 16;
    const std::vector<int32_t> &ab = c.abmn_h;
    auto col = [&](int32_t e) { return e < 0 ? c.nE : e; };
    std::vector<StiffChunk> chunks;
    std::vector<int32_t> dipa, dipm;
    std::vector<int4> meta;
    meta.reserve((size_t)c.D);
    size_t tab_max = 0;
    int64_t d = 0;
    while (d < c.D) {
        std::map<std::pair<int32_t, int32_t>, int32_t> amap, mmap;
        std::vector<std::array<int32_t, 3>> rows;  // (ia, d, im) of the chunk
        const int64_t d0 = d;
        for (; d < c.D; d++) {
            const int32_t *q = &ab[4 * d];
            const int na = (int)amap.size() + (amap.count({q[0], q[1]}) ? 0 : 1);
            const int nmm = (int)mmap.size() + (mmap.count({q[2], q[3]}) ? 0 : 1);
            if ((size_t)(na + nmm) * per_dip > tab_cap || na > 65535 || nmm > 32767) {
                if (d == d0) return;  // one datum does not fit: no plan
                break;
            }
            const int32_t ia = amap.emplace(std::make_pair(q[0], q[1]), (int32_t)amap.size()).first->second;
            const int32_t im = mmap.emplace(std::make_pair(q[2], q[3]), (int32_t)mmap.size()).first->second;
            rows.push_back({ia, (int32_t)d, im});
        }
        StiffChunk cd{};
        cd.s0 = (int32_t)meta.size();
        cd.s1 = cd.s0 + (int32_t)rows.size();
        cd.nA = (int32_t)amap.size();
        cd.nM = (int32_t)mmap.size();
        cd.off_a = (int32_t)(dipa.size() / 2);
        cd.off_m = (int32_t)(dipm.size() / 2);
        tab_max = std::max(tab_max, (size_t)(cd.nA + cd.nM) * per_dip);
        std::vector<int32_t> da(2 * amap.size()), dm(2 * mmap.size());
        for (auto &kv : amap) {
            da[2 * kv.second] = col(kv.first.first);
            da[2 * kv.second + 1] = col(kv.first.second);
        }
        for (auto &kv : mmap) {
            dm[2 * kv.second] = col(kv.first.first);
            dm[2 * kv.second + 1] = col(kv.first.second);
        }
        dipa.insert(dipa.end(), da.begin(), da.end());
        dipm.insert(dipm.end(), dm.begin(), dm.end());
        std::sort(rows.begin(), rows.end());
        for (auto &r : rows) {
            // (datum, ia | im << 16, geometric factor: FP32 bits in .z or FP64 bits in .z/.w)
            const double kf = c.kfac_h[r[1]];
            int4 rec = make_int4(r[1], r[0] | (r[2] << 16), 0, 0);
            if (dt == 1) {
                const float f = (float)kf;
                std::memcpy(&rec.z, &f, 4);
            } else {
                std::memcpy(&rec.z, &kf, 8);
            }
            meta.push_back(rec);
        }
        chunks.push_back(cd);
    }
    S.RS = RS;
    S.tab_bytes = (tab_max + 15) / 16 * 16;
    S.stage_bytes = stage;
    S.smem = S.tab_bytes + stage + fixed;
    S.nchunks = (int)chunks.size();
    S.d_pc.upload(pc, c.stream);
    S.d_nptr.upload(nptr, c.stream);
    S.d_tnodes.upload(tnodes, c.stream);
    S.d_lidx.upload(lidx, c.stream);
    S.d_dipa.upload(dipa, c.stream);
    S.d_dipm.upload(dipm, c.stream);
    std::vector<int32_t> cw(chunks.size() * 12);
    std::memcpy(cw.data(), chunks.data(), cw.size() * sizeof(int32_t));
    S.d_chunks.upload(cw, c.stream);
    std::vector<int32_t> mw(meta.size() * 4);
    std::memcpy(mw.data(), meta.data(), mw.size() * sizeof(int32_t));
    S.d_meta.upload(mw, c.stream);
    ERTGB_CUDA(cudaStreamSynchronize(c.stream));  // host lists are freed on return
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
